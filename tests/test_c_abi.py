"""The C ABI from C: tests/c_abi/solve_2d.c is compiled with gcc against
include/dcrf.h and linked with the engine's shared library, as a host binding
the library directly would.  On a machine without a GPU the program must get
an explicit DCRF_ERR_NO_DEVICE; with a GPU it solves a small image and checks
the marginals, dcrf_map and run-to-run reproducibility."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "pydensecrf_gb300")


def _build(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    if not os.path.exists(os.path.join(LIBDIR, "libdcrf_gb300.so")):
        pytest.fail("libdcrf_gb300.so is missing: build the engine first")
    exe = str(tmp_path / "solve_2d")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_abi", "solve_2d.c"), "-o", exe, "-L", LIBDIR, "-ldcrf_gb300",
                    "-Wl,-rpath," + LIBDIR, "-lm"], check=True)
    return exe


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_c_program_without_device_gets_explicit_error(tmp_path):
    if _has_gpu():
        pytest.skip("a GPU is visible")
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines()[0] == "abi 1"
    assert "no device" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("args", [("64", "48", "5", "5"), ("37", "21", "21", "10")])
def test_c_program_solves_on_device(tmp_path, args):
    exe = _build(tmp_path)
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert "map ok, repeat identical" in r.stdout, r.stdout
