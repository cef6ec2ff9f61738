"""The reference-side binding a maintainer would add: the Cython extension
tests/cython_binding/densecrf_cy.pyx (the reference's DenseCRF / DenseCRF2D
classes over the engine's C ABI) is cythonized, compiled with gcc against
include/dcrf.h, linked with the engine's shared library and imported.  Without
a GPU every handle creation must fail with an explicit error (no CPU path); the
argument checks run on the host and raise the reference's exception types."""
import os
import shutil
import subprocess
import sys
import sysconfig

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "pydensecrf_gb300")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def extdir(tmp_path_factory):
    pytest.importorskip("Cython")
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    if not os.path.exists(os.path.join(LIBDIR, "libdcrf_gb300.so")):
        pytest.fail("libdcrf_gb300.so is missing: build the engine first")
    out = tmp_path_factory.mktemp("cy")
    c_file = str(out / "densecrf_cy.c")
    subprocess.run([sys.executable, "-m", "cython", "-3", os.path.join(ROOT, "tests", "cython_binding",
                                                                      "densecrf_cy.pyx"), "-o", c_file], check=True)
    so = str(out / ("densecrf_cy" + sysconfig.get_config_var("EXT_SUFFIX")))
    subprocess.run(["gcc", "-O1", "-shared", "-fPIC", "-I", sysconfig.get_paths()["include"], "-I",
                    os.path.join(ROOT, "include"), c_file, "-L", LIBDIR, "-ldcrf_gb300", "-Wl,-rpath," + LIBDIR,
                    "-o", so], check=True)
    return str(out)


def _run(extdir, code):
    r = subprocess.run([sys.executable, "-c", "import densecrf_cy as d, numpy as np\n" + code], cwd=extdir,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_binding_loads_and_reports_abi(extdir):
    assert _run(extdir, "print(d.abi_version())").strip() == "1"


def test_binding_without_device_raises(extdir):
    if _has_gpu():
        pytest.skip("a GPU is visible")
    out = _run(extdir, """
for make in (lambda: d.DenseCRF(100, 2), lambda: d.DenseCRF2D(10, 10, 2)):
    try:
        make()
        print("created")
    except RuntimeError as e:
        print("RuntimeError", e)
""")
    assert out.splitlines() == ["RuntimeError no CUDA device available"] * 2


def test_binding_compatibility_dispatch(extdir):
    out = _run(extdir, """
k, v = d.compat_buffer(3, 4); print(k, v.tolist())
k, v = d.compat_buffer(np.arange(4, dtype=np.float32), 4); print(k, v.tolist())
k, v = d.compat_buffer(np.eye(2, dtype=np.float32), 2); print(k, v.shape)
for bad in (np.ones(4), np.ones((2, 2, 2), np.float32), np.ones(3, np.float32)):
    try:
        d.compat_buffer(bad, 4)
        print("accepted")
    except ValueError:
        print("ValueError")
""")
    assert out.splitlines() == ["0 [3.0]", "1 [0.0, 1.0, 2.0, 3.0]", "2 (2, 2)", "ValueError", "ValueError",
                                "ValueError"]
