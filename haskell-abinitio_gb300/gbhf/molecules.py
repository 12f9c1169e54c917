"""Seeded synthetic water clusters and the single-water test geometry.

No public benchmark set exists for the reference (it publishes no numbers), so
the workloads are seeded water clusters:

* monomer r(OH) = 0.9572 A, angle HOH = 104.52 deg, atom order O, H, H;
* sites on a 3.0 A cubic grid, the first n sites of the smallest k^3 >= n cube
  in lexicographic (i, j, k) order;
* per monomer a uniform random rotation (Shoemake's quaternion construction)
  and a uniform +-0.3 A translation jitter on each axis; the monomer is drawn
  again while any O-O distance to an already placed monomer is below 2.6 A;
* ``numpy.random.default_rng(seed)``; Angstrom -> bohr by dividing by
  0.529177 as ``angstrom2AU`` does (Units.hs:12-13).

Because libm trigonometry may differ in the last bit between machines, the
generated clusters are committed in ``data/water_clusters.json`` (made by
``write_cluster_file``) and the workloads read that file.
"""
from __future__ import annotations

import json
import math
from functools import lru_cache
from pathlib import Path

import numpy as np

from .basis import ANGSTROM_TO_BOHR, make_atoms

R_OH = 0.9572
THETA_HOH = math.radians(104.52)
GRID = 3.0
JITTER = 0.3
MIN_OO = 2.6

# Workload seeds: (H2O)16 -> 0, (H2O)8 -> 1, 256 conformers -> 2, (H2O)64 -> 3.
SEEDS = {"w16": 0, "w8": 1, "batch256": 2, "w64": 3}

# Single water, bohr: O (0,0,0); H (0,+-1.4305,1.1093).
WATER_BOHR = np.array([[0.0, 0.0, 0.0], [0.0, 1.4305, 1.1093], [0.0, -1.4305, 1.1093]])


def _monomer():
    h = R_OH
    s, c = math.sin(THETA_HOH / 2), math.cos(THETA_HOH / 2)
    return np.array([[0.0, 0.0, 0.0], [h * s, 0.0, h * c], [-h * s, 0.0, h * c]])


def _rotation(u):
    """Shoemake (1992) uniform quaternion from three uniforms -> rotation matrix."""
    u1, u2, u3 = u
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2),
                  math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3),
                  math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    x, y, z, w = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _sites(n):
    k = 1
    while k ** 3 < n:
        k += 1
    out = [(i, j, l) for i in range(k) for j in range(k) for l in range(k)]
    return np.array(out[:n], dtype=np.float64) * GRID


def water_cluster(n, rng):
    """Coordinates (3n, 3) in bohr of a seeded (H2O)_n cluster."""
    mono = _monomer()
    placed_o = []
    atoms = []
    for site in _sites(n):
        while True:
            rot = _rotation(rng.random(3))
            shift = site + rng.uniform(-JITTER, JITTER, size=3)
            xyz = mono @ rot.T + shift
            if all(np.linalg.norm(xyz[0] - o) >= MIN_OO for o in placed_o):
                break
        placed_o.append(xyz[0])
        atoms.append(xyz)
    return np.concatenate(atoms, axis=0) * ANGSTROM_TO_BOHR


def generate_all():
    out = {}
    for name, n in (("w16", 16), ("w8", 8), ("w64", 64)):
        out[name] = water_cluster(n, np.random.default_rng(SEEDS[name])).tolist()
    rng = np.random.default_rng(SEEDS["batch256"])
    sizes = [int(v) for v in rng.integers(1, 13, size=256)]
    out["batch256"] = [water_cluster(n, rng).tolist() for n in sizes]
    return out


def write_cluster_file(path=None):
    path = Path(path) if path else Path(__file__).with_name("data") / "water_clusters.json"
    data = generate_all()
    path.write_text(json.dumps({k: v for k, v in data.items()}, separators=(",", ":")))
    return path


@lru_cache(maxsize=None)
def _cluster_file():
    return json.loads((Path(__file__).with_name("data") / "water_clusters.json").read_text())


def cluster_coords(name, index=None):
    d = _cluster_file()[name]
    return np.asarray(d if index is None else d[index], dtype=np.float64)


def water_labels(n_waters):
    return ["O", "H", "H"] * n_waters


def water_atoms(basis="sto-3g", variant="text"):
    """The single-water workload (bohr geometry above)."""
    return make_atoms(["O", "H", "H"], WATER_BOHR, basis, variant)


def cluster_atoms(name, basis="6-31g", variant="text", index=None):
    xyz = cluster_coords(name, index)
    return make_atoms(water_labels(len(xyz) // 3), xyz, basis, variant)


def batch_workload(variant="text"):
    """The 256-conformer batch: STO-3G for even index, 6-31G for odd index."""
    confs = _cluster_file()["batch256"]
    return [make_atoms(water_labels(len(c) // 3), c, "sto-3g" if i % 2 == 0 else "6-31g", variant)
            for i, c in enumerate(confs)]


if __name__ == "__main__":
    print(write_cluster_file())


def _small_geometries():
    """Small molecules over the elements of the basis data (H-Ne), bohr;
    approximate experimental bond lengths, charge of the molecule."""
    s3 = math.sqrt(3.0)
    r_nh, a_nh = 1.913, math.radians(106.7)
    # NH3: N on the axis, the three H on a cone (H-N-H angle a_nh)
    hx = r_nh * math.sqrt(2 * (1 - math.cos(a_nh)) / 3)
    hz = -math.sqrt(r_nh ** 2 - hx ** 2)
    nh3 = [("N", (0.0, 0.0, 0.0))] + [("H", (hx * math.cos(t), hx * math.sin(t), hz))
                                      for t in (0.0, 2 * math.pi / 3, 4 * math.pi / 3)]
    r_ch = 2.052 / s3
    ch4 = [("C", (0.0, 0.0, 0.0)), ("H", (r_ch, r_ch, r_ch)), ("H", (-r_ch, -r_ch, r_ch)),
           ("H", (-r_ch, r_ch, -r_ch)), ("H", (r_ch, -r_ch, -r_ch))]
    r_bh = 2.25
    bh3 = [("B", (0.0, 0.0, 0.0))] + [("H", (r_bh * math.cos(t), r_bh * math.sin(t), 0.0))
                                      for t in (0.0, 2 * math.pi / 3, 4 * math.pi / 3)]
    return {
        "CO": ([("C", (0.0, 0.0, 0.0)), ("O", (0.0, 0.0, 2.132))], 0.0),
        "HF": ([("F", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.733))], 0.0),
        "NH3": (nh3, 0.0),
        "CH4": (ch4, 0.0),
        "BH3": (bh3, 0.0),
        "LiH": ([("Li", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 3.015))], 0.0),
        "BeH2": ([("Be", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 2.54)), ("H", (0.0, 0.0, -2.54))], 0.0),
        "Ne": ([("Ne", (0.0, 0.0, 0.0))], 0.0),
        "HHe+": ([("H", (0.0, 0.0, 0.0)), ("He", (0.0, 0.0, 1.4632))], 1.0),
    }


def small_molecule(name, basis="sto-3g", variant="text"):
    """(atoms, charge) of one of the small test molecules (``_small_geometries``)."""
    geo, charge = _small_geometries()[name]
    labels = [l for l, _ in geo]
    return make_atoms(labels, [xyz for _, xyz in geo], basis, variant), charge


SMALL_MOLECULES = ("CO", "HF", "NH3", "CH4", "BH3", "LiH", "BeH2", "Ne", "HHe+")


def _open_shell_geometries():
    """Open-shell test systems: (atoms (label, bohr), charge, multiplicity)."""
    def bent(center, r, angle_deg):
        t = math.radians(angle_deg) / 2
        return [(center, (0.0, 0.0, 0.0)), ("H", (0.0, r * math.sin(t), r * math.cos(t))),
                ("H", (0.0, -r * math.sin(t), r * math.cos(t)))]
    return {
        "H": ([("H", (0.0, 0.0, 0.0))], 0.0, 2),
        "Li": ([("Li", (0.0, 0.0, 0.0))], 0.0, 2),
        "OH": ([("O", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.834))], 0.0, 2),
        "NH2": (bent("N", 1.936, 103.0), 0.0, 2),
        "CH2": (bent("C", 2.04, 134.0), 0.0, 3),
        "O2": ([("O", (0.0, 0.0, 0.0)), ("O", (0.0, 0.0, 2.282))], 0.0, 3),
        "H2O+": ([("O", tuple(WATER_BOHR[0])), ("H", tuple(WATER_BOHR[1])), ("H", tuple(WATER_BOHR[2]))], 1.0, 2),
    }


def open_shell_molecule(name, basis="sto-3g", variant="text"):
    """(atoms, charge, multiplicity) of an open-shell test system."""
    geo, charge, mult = _open_shell_geometries()[name]
    return make_atoms([l for l, _ in geo], [x for _, x in geo], basis, variant), charge, mult


OPEN_SHELL = ("H", "Li", "OH", "NH2", "CH2", "O2", "H2O+")
