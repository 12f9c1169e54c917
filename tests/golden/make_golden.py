"""Generate the golden fixtures in this directory.

Run from the repository root:  python tests/golden/make_golden.py

* ``quadrature256.json``: SHA-256 of the reference's 256-point Gauss-Legendre
  table (points256/weights256 in
  Science/QuantumChemistry/NumericalTools/PointsWeights.hs, parsed as
  float64, big-endian) and how far the oracle's own nodes/weights lie from it.
  Needs the reference checkout (REFERENCE_ROOT, default /root/reference).
* ``water_sto3g.json``: single water (O (0,0,0); H (0,+-1.4305,1.1093) bohr),
  STO-3G, for both basis variants (as shipped = SP exponents 1.0, and the
  EMSL text): overlap, core Hamiltonian and the canonical ERI array in both
  numerics presets, and the SCF energies of the oracle driver.
* ``clusters.json``: oracle SCF energies (exact numerics, direct build,
  Schwarz 1e-12) of the (H2O)_2 6-31G and (H2O)_4 STO-3G clusters taken from
  the seeded 256-conformer set (indices documented in the file).
The data are oracle outputs; the oracle itself is pinned by the reference's
known-answer data (tests/test_oracle_*.py).
"""
import hashlib
import json
import os
import re
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "haskell-abinitio_gb300"))
import oracle as O  # noqa: E402
from gbhf import basis as B, molecules as M  # noqa: E402

OUT = Path(__file__).resolve().parent
REF = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))


def table_hash(x, w):
    return hashlib.sha256(np.asarray(x, ">f8").tobytes() + np.asarray(w, ">f8").tobytes()).hexdigest()


def quadrature():
    src = (REF / "Science/QuantumChemistry/NumericalTools/PointsWeights.hs").read_text()

    def get(name):
        m = re.search(name + r" = U.fromList \[([^\]]*)\]", src)
        return np.array([float(v) for v in m.group(1).split(",")])

    px, pw = get("points256"), get("weights256")
    x, w = O.gauss_legendre(256)
    return {"reference_sha256": table_hash(px, pw),
            "n_positive_nodes": int(px.size),
            "max_abs_node_diff": float(np.max(np.abs(x - px))),
            "max_abs_weight_diff": float(np.max(np.abs(w - pw))),
            "weights_differing": int(np.sum(w != pw))}


def water():
    out = {"geometry_bohr": M.WATER_BOHR.tolist()}
    for variant in ("shipped", "text"):
        fb = B.flatten(M.water_atoms("sto-3g", variant))
        ob = O.OracleBasis(fb)
        d = {}
        for ref in (True, False):
            key = "reference" if ref else "exact"
            d[key] = {"overlap": ob.overlap(ref).tolist(), "hcore": ob.hcore(ref).tolist(),
                      "eri": ob.eri_canonical(ref).tolist()}
        d["energy_reference_driver"] = O.scf(fb, O.SCFOptions.reference()).energy
        d["energy_baseline_driver"] = O.scf(fb, O.SCFOptions.baseline()).energy
        out[variant] = d
    return out


def clusters():
    confs = M._cluster_file()["batch256"]
    # first conformers with 2 and 4 waters, 6-31G (odd index) and STO-3G (even index)
    pick = {}
    for i, c in enumerate(confs):
        nw = len(c) // 3
        if nw == 2 and i % 2 == 1 and "w2_631g" not in pick:
            pick["w2_631g"] = (i, "6-31g")
        if nw == 4 and i % 2 == 0 and "w4_sto3g" not in pick:
            pick["w4_sto3g"] = (i, "sto-3g")
    out = {}
    for name, (i, bas) in pick.items():
        fb = B.flatten(M.cluster_atoms("batch256", bas, "text", index=i))
        r = O.scf(fb, O.SCFOptions.baseline())
        rs = O.scf(fb, O.SCFOptions.baseline(guess="sad"))
        out[name] = {"batch_index": i, "basis": bas, "energy": r.energy, "iterations": r.iterations,
                     "energy_sad": rs.energy, "iterations_sad": rs.iterations, "n_basis": int(fb.n_cgf)}
    # (H2O)16 6-31G: minutes on 8 cores; the entries already in the previous
    # file are kept unless GOLDEN_W16=1
    prev = OUT / "clusters.json"
    old = json.loads(prev.read_text()) if prev.exists() else {}
    rec = old.get("w16_631g", {})
    fb = B.flatten(M.cluster_atoms("w16", "6-31g"))
    if os.environ.get("GOLDEN_W16") == "1" or "energy" not in rec:
        r = O.scf(fb, O.SCFOptions.baseline())
        rec = {"cluster": "w16", "basis": "6-31g", "energy": r.energy, "iterations": r.iterations,
               "n_basis": int(fb.n_cgf)}
    if os.environ.get("GOLDEN_W16") == "1" or "iterations_sad" not in rec:
        rs = O.scf(fb, O.SCFOptions.baseline(guess="sad"))
        rec.update(energy_sad=rs.energy, iterations_sad=rs.iterations)
    out["w16_631g"] = rec
    return out


def main():
    if REF.exists():
        (OUT / "quadrature256.json").write_text(json.dumps(quadrature(), indent=1) + "\n")
    (OUT / "water_sto3g.json").write_text(json.dumps(water()) + "\n")
    (OUT / "clusters.json").write_text(json.dumps(clusters(), indent=1) + "\n")


if __name__ == "__main__":
    main()
