"""Generate the golden fixtures in this directory.

Run from the repository root:  python tests/golden/make_golden.py

* ``quadrature256.json``: SHA-256 of the reference's 256-point Gauss-Legendre
  table (points256/weights256 in
  Science/QuantumChemistry/NumericalTools/PointsWeights.hs, parsed as
  float64, big-endian) and how far the oracle's own nodes/weights lie from it.
  Needs the reference checkout, given as the first argument or by the
  REFERENCE_ROOT environment variable.
* ``sample_projects.json``: the literal primitives and geometries of the
  reference's four sample projects (HsFock/SampleProjects.hs:18-98: HHe+,
  CO and water in STO-3G, water in 6-31G*), parsed from that file, with the
  oracle's energies on exactly those inputs.  Needs the reference checkout.
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
_ref_arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT", "")
REF = Path(_ref_arg) if _ref_arg else None


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


# Atom of each entry of ``atomList`` (HsFock/SampleProjects.hs).  The
# reference's own test pairs "water" as O, H, H with [baseH, baseO] = pBasis
# (test/AbinitioTests.hs:16-22); HHe+ and CO have no caller and pair pBasis
# with atomList in order.  Charges: HHe+ is a cation.
SAMPLE_ATOMS = {("HHe+", "STO-3G"): (["He", "H"], 1.0), ("CO", "STO-3G"): (["O", "C"], 0.0),
                ("water", "STO-3G"): (["O", "H", "H"], 0.0), ("water", "6-31G*"): (["O", "H", "H"], 0.0)}
SAMPLE_BASE = {"H": "baseH", "He": "baseHe", "C": "baseC", "O": "baseO"}
ZNUM = {"H": 1.0, "He": 2.0, "C": 6.0, "O": 8.0}


def _hs_float(tok):
    return float(tok.strip())


def sample_projects():
    """Parse project "<label>" "<basis>" = PD {...} where ... blocks."""
    src = (REF / "Science/QuantumChemistry/HsFock/SampleProjects.hs").read_text()
    heads = list(re.finditer(r'^project "([^"]+)" "([^"]+)" *=', src, flags=re.M))
    out = {}
    for k, m in enumerate(heads):
        body = src[m.end():heads[k + 1].start() if k + 1 < len(heads) else len(src)]
        atoms_txt = re.search(r"atomList\s*=\s*\[(.*?)\]\s*\}", body, flags=re.S).group(1)
        coords = [[_hs_float(v) for v in t.split(",")] for t in re.findall(r"\[([^\[\]]+)\]", atoms_txt)]
        prims = {}
        for name, lst in re.findall(r"^\s*(\w+)\s*=\s*\[\s*(\([^=]*?\))\s*\]\s*$", body, flags=re.M):
            prims[name] = [[_hs_float(c), _hs_float(e)] for c, e in re.findall(r"\(([^,()]+),([^,()]+)\)", lst)]
        bases = {}
        for name, lst in re.findall(r"^\s*(base\w+)\s*=\s*normGlobal`fmap`\s*\[(.*?)\]\s*$", body, flags=re.M):
            bases[name] = [{"primitives": prims[pn], "funtype": ft}
                           for pn, ft in re.findall(r"CGF\s+(\w+)\s+(\w+)", lst)]
        labels, charge = SAMPLE_ATOMS[(m.group(1), m.group(2))]
        assert len(labels) == len(coords)
        rec = {"label": m.group(1), "basis": m.group(2), "charge": charge,
               "atoms": [{"element": l, "znumber": ZNUM[l], "coord_bohr": c, "cgfs": bases[SAMPLE_BASE[l]]}
                         for l, c in zip(labels, coords)]}
        fb = B.flatten(sample_atoms(rec))
        occ_opts = dict(charge=charge)
        rec["oracle_energy_exact"] = O.scf(fb, O.SCFOptions.baseline(guess="sad", **occ_opts)).energy
        try:
            rec["oracle_energy_reference"] = O.scf(fb, O.SCFOptions(charge=charge)).energy
        except IndexError as e:   # the Harris guess leaves the ERI array (as the reference would)
            rec["oracle_energy_reference"] = None
            rec["reference_driver_error"] = str(e)
        out[f"{m.group(1)} {m.group(2)}"] = rec
    return out


def sample_atoms(rec):
    """``[AtomData]`` of a sample project: the literal primitives through
    ``normGlobal`` (``basis.norm_coeff``), in the project's own CGF order."""
    atoms = []
    for a in rec["atoms"]:
        cgfs = []
        for c in a["cgfs"]:
            cs = [p[0] for p in c["primitives"]]
            es = [p[1] for p in c["primitives"]]
            cgfs.append(B.CGF(tuple(zip(B.norm_coeff(c["funtype"], cs, es), es)), c["funtype"]))
        atoms.append(B.AtomData(tuple(a["coord_bohr"]), cgfs, a["znumber"], a["element"]))
    return atoms


def main():
    if REF is not None and REF.exists():
        (OUT / "quadrature256.json").write_text(json.dumps(quadrature(), indent=1) + "\n")
        (OUT / "sample_projects.json").write_text(json.dumps(sample_projects(), indent=1) + "\n")
    else:
        print("no reference checkout given (argument or REFERENCE_ROOT): "
              "quadrature256.json and sample_projects.json are kept as they are")
    (OUT / "water_sto3g.json").write_text(json.dumps(water()) + "\n")
    (OUT / "clusters.json").write_text(json.dumps(clusters(), indent=1) + "\n")


if __name__ == "__main__":
    main()
