"""The C++ plugin-class mirror (include/pimc_gb300.hpp) used as a drop-in:
tests/cpp/dropin.cpp is compiled with g++ against the library and the oracle.
On a machine without a GPU it must throw pgb::Error(PGB_ECUDA); on the GPU
every action, per-slice term and estimator it returns must match the oracle."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def dropin(pgb, oracle_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("cpp") / "dropin")
    libdir = os.path.dirname(pgb._lib.LIB_PATH)
    odir = os.path.join(ROOT, "oracle", "_build")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
           os.path.join(ROOT, "tests", "cpp", "dropin.cpp"), "-o", exe,
           "-L", libdir, "-l:libpimc_gb300.so", "-L", odir, "-l:libpimc_oracle.so",
           "-Wl,-rpath," + libdir, "-Wl,-rpath," + odir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_header_compiles_standalone(tmp_path):
    src = tmp_path / "only.cpp"
    src.write_text('#include "pimc_gb300.hpp"\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_dropin_throws_without_device(dropin):
    r = subprocess.run([dropin, "nodevice"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "code -2" in r.stdout


@pytest.mark.gpu
def test_dropin_parity(dropin):
    r = subprocess.run([dropin, "parity"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "mismatches 0" in r.stdout
