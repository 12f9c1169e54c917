"""The generated gradient code is the derivative of the generated ERI code.

``tests/host/grad_fd_check.cpp`` compiles ``csrc/eri_gen.cuh`` and
``csrc/grad_gen.cuh`` for the host and compares, for eight classes ((ss|ss)
through (pp|pp), and (ds|ss), (ds|ps)), the generated bra-centre derivatives
of one primitive quartet contracted with a random Gamma against central
differences of the generated ERIs (h = 1e-4 bohr: truncation error ~1e-8 of
the largest derivative).  No GPU: this checks the generators' algebra (the
derivative rule of the basis functions, HartreeFock/Derivatives.hs:246-257, in
Hermite form) before any device runs it."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "haskell-abinitio_gb300" / "csrc"
SRC = Path(__file__).resolve().parent / "host" / "grad_fd_check.cpp"


def test_generated_gradient_matches_finite_differences_of_generated_eris(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "grad_fd_check"
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", str(CSRC), str(SRC), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    res = dict(zip(out[0::2], map(float, out[1::2])))
    assert set(res) == {"ssss", "psss", "psps", "sspp", "pspp", "pppp", "dsss", "dsps"}
    for cls, err in res.items():
        assert err < 1e-6, (cls, err)
