"""The reference-side binding a maintainer would add: the Cython extension
tests/cython_binding/densecrf_cy.pyx (the reference's DenseCRF / DenseCRF2D
classes over the engine's C ABI) is cythonized, compiled with gcc against
include/dcrf.h, linked with the engine's shared library and imported.  Without
a GPU every handle creation must fail with an explicit error (no CPU path); the
argument checks run on the host and raise the reference's exception types.  On
a GPU the binding solves the reference's golden cases (inference,
startInference + stepInference, klDivergence) to the golden's tolerances.

Where Cython itself is not installed (the GPU hosts), the C file that the
engine's build generated from the .pyx (tests/cython_binding/_gen/, made by
__graft_entry__.build() wherever Cython is present) is compiled instead."""
import os
import shutil
import subprocess
import sys
import sysconfig

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "pydensecrf_gb300")
PYX = os.path.join(ROOT, "tests", "cython_binding", "densecrf_cy.pyx")
GENERATED = os.path.join(ROOT, "tests", "cython_binding", "_gen", "densecrf_cy.c")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def extdir(tmp_path_factory):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    if not os.path.exists(os.path.join(LIBDIR, "libdcrf_gb300.so")):
        pytest.fail("libdcrf_gb300.so is missing: build the engine first")
    out = tmp_path_factory.mktemp("cy")
    c_file = str(out / "densecrf_cy.c")
    try:
        import Cython  # noqa: F401
        subprocess.run([sys.executable, "-m", "cython", "-3", PYX, "-o", c_file], check=True)
    except ImportError:
        if not os.path.exists(GENERATED):
            pytest.skip("neither Cython nor a C file generated from the .pyx is available")
        shutil.copy(GENERATED, c_file)
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


@pytest.mark.gpu
def test_binding_solves_reference_golden(extdir):
    """Through the Cython binding alone: the reference's golden marginals after
    T iterations, one startInference + stepInference, and klDivergence
    (densecrf.pyx:91-101), for a Potts, a Diagonal and a Matrix case."""
    if not _has_gpu():
        pytest.fail("GPU test collected but no CUDA device is visible")
    golden = os.path.join(ROOT, "tests", "golden", "inference.npz")
    out = _run(extdir, f"""
g = np.load({golden!r})
W, H, M, T = int(g["W"]), int(g["H"]), int(g["M"]), int(g["T"])
compat = {{"potts": 3.0, "diag": g["diag"], "mat": g["mat"]}}
for name in ("potts_n3", "diag_n2", "mat_n1"):
    ck, nt = name.split("_n")
    c = d.DenseCRF2D(W, H, M)
    c.setUnaryEnergy(np.ascontiguousarray(g["U"].T))
    c.addPairwiseGaussian(3.0, compat[ck], d.DIAG_KERNEL, int(nt))
    c.addPairwiseBilateral(8.0, 13.0, np.ascontiguousarray(g["img"]), 5.0)
    Q = c.inference(T)
    e_q = float(np.abs(Q.T - g[name + "/sse/Q"]).max())
    Q1 = c.startInference()
    e_0 = float(np.abs(Q1.T - g["Q0"]).max())
    c.stepInference(Q1)
    e_1 = float(np.abs(Q1.T - g[name + "/sse/Q1"]).max())
    kl = c.klDivergence(np.ascontiguousarray(g[name + "/sse/Q"].T))
    kl_ref = float(g[name + "/sse/kl"])
    print(name, e_q, e_0, e_1, abs(kl - kl_ref) / max(1.0, abs(kl_ref)))
""")
    lines = out.strip().splitlines()
    assert len(lines) == 3, out
    for ln in lines:
        name, e_q, e_0, e_1, e_kl = ln.split()
        assert float(e_q) < 1e-4 and float(e_0) < 1e-6 and float(e_1) < 1e-4, ln
        assert float(e_kl) <= 1e-5, ln
