"""The generated integral code on the host: the ERIs against the oracle, and
the gradient code as the derivative of the ERI code.

``tests/host/grad_fd_check.cpp`` compiles ``csrc/eri_gen.cuh`` and
``csrc/grad_gen.cuh`` for the host and compares, for all 14 generated classes
(the s/p ones and the light d ones), the generated bra-centre derivatives
of one primitive quartet contracted with a random Gamma against central
differences of the generated ERIs (h = 1e-4 bohr: truncation error ~1e-8 of
the largest derivative).  No GPU: this checks the generators' algebra (the
derivative rule of the basis functions, HartreeFock/Derivatives.hs:246-257, in
Hermite form) before any device runs it.  ``tests/host/eri_oracle_check.cpp``
does the same for the ERIs themselves: one primitive per shell, the thirteen
generated classes (six s/p, seven d), against the oracle's contracted ERIs in
exact numerics."""
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
    assert set(res) == {"ssss", "psss", "psps", "sspp", "pspp", "pppp", "dsss", "dsps",
                        "ssps", "ppss", "ppps", "ssds", "ssdp", "psds"}
    for cls, err in res.items():
        assert err < 1e-6, (cls, err)


CLASSES = {"ssss": (0, 0, 0, 0), "psss": (1, 0, 0, 0), "psps": (1, 0, 1, 0), "sspp": (0, 0, 1, 1),
           "pspp": (1, 0, 1, 1), "pppp": (1, 1, 1, 1), "dsss": (2, 0, 0, 0), "dsps": (2, 0, 1, 0),
           "dspp": (2, 0, 1, 1), "dsds": (2, 0, 2, 0), "dpss": (2, 1, 0, 0), "dpps": (2, 1, 1, 0),
           "ddss": (2, 2, 0, 0)}
LABELS = {0: ("S",), 1: ("Px", "Py", "Pz"), 2: ("Dxx", "Dxy", "Dxz", "Dyy", "Dyz", "Dzz")}


def test_generated_eris_match_the_oracle(tmp_path):
    """eri_ketprim_<class> for one primitive per shell against the oracle's
    contracted ERIs (exact numerics) of the same one-primitive functions, for
    the six s/p classes and the seven lane-per-ket d classes, 1e-12 relative to
    the largest integral."""
    import numpy as np
    import oracle as O
    from gbhf import basis as B
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "eri_oracle_check"
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", str(CSRC), str(SRC.parent / "eri_oracle_check.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    rng = np.random.default_rng(5)
    worst = 0.0
    for cls, ls in CLASSES.items():
        for rep in range(3):
            xyz = rng.uniform(-1.2, 1.2, (4, 3))
            ex = rng.uniform(0.3, 2.0, 4)
            co = rng.uniform(0.5, 1.5, 4)
            atoms = []
            for k in range(4):
                fns = [B.CGF(((co[k], ex[k]),), t) for t in LABELS[ls[k]]]
                atoms.append(B.AtomData(tuple(xyz[k]), fns, 1.0))
            ob = O.OracleBasis(B.flatten(atoms))
            first = np.cumsum([0] + [len(LABELS[l]) for l in ls])
            line = " ".join([cls] + [f"{v:.17e}" for v in xyz.ravel()] + [f"{v:.17e}" for v in ex] +
                            [f"{v:.17e}" for v in co])
            got = np.array(subprocess.run([str(exe)], input=line + "\n", check=True, capture_output=True,
                                          text=True).stdout.split(), dtype=float)
            ref = []
            for ia in range(len(LABELS[ls[0]])):
                for ib in range(len(LABELS[ls[1]])):
                    for ic in range(len(LABELS[ls[2]])):
                        for id_ in range(len(LABELS[ls[3]])):
                            ref.append(ob.eri(first[0] + ia, first[1] + ib, first[2] + ic, first[3] + id_,
                                              ref_compat=False))
            ref = np.array(ref)
            assert got.shape == ref.shape, cls
            err = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300)
            worst = max(worst, err)
            assert err < 1e-12, (cls, err)
    print(f"worst relative difference {worst:.2e}")
    assert worst < 1e-12
