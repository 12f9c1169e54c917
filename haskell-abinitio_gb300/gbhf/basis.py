"""Basis-set types and CGF construction, mirroring the reference's boundary types.

``AtomData``/``CGF`` follow ``Science.QuantumChemistry.GlobalTypes``
(GlobalTypes.hs:92-105): an atom is (coordinates in bohr, list of contracted
Gaussian functions, nuclear charge); a CGF is a list of primitives
``(coefficient, exponent)`` plus a Cartesian label.

``create_cgf`` restates ``createCGF`` (BasisSet/FetchBasis.hs:50-59): an SP
shell becomes S, Px, Py, Pz (sharing exponents), a P shell Px, Py, Pz and a D
shell Dxx, Dxy, Dxz, Dyy, Dyz, Dzz.  Every CGF then goes through
``normGlobal`` (BasisSet/NormalizeBasis.hs:37-59), which multiplies each
coefficient by the Cartesian primitive normalisation and then by
``sqrt(1/S_cgf,cgf)``.  In the reference that last factor is always 1.0
because ``sijContracted`` returns 1.0 for identical CGFs on one centre
(Integrals/IntegralsEvaluation.hs:183-184), so contracted functions stay
unnormalised; ``create_cgf`` keeps that behaviour.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from functools import lru_cache
from pathlib import Path
from typing import List, Sequence, Tuple

import numpy as np

ANGSTROM_TO_BOHR = 1.0 / 0.529177  # Units.hs:12-13 divides by 0.529177

# Cartesian exponents per label (GlobalTypes.hs:263-284 ``mapLAngular``).
FUNTYPES = {
    "S": (0, 0, 0),
    "Px": (1, 0, 0), "Py": (0, 1, 0), "Pz": (0, 0, 1),
    "Dxx": (2, 0, 0), "Dxy": (1, 1, 0), "Dxz": (1, 0, 1),
    "Dyy": (0, 2, 0), "Dyz": (0, 1, 1), "Dzz": (0, 0, 2),
}
SHELL_LABELS = {
    "S": ("S",),
    "P": ("Px", "Py", "Pz"),
    "D": ("Dxx", "Dxy", "Dxz", "Dyy", "Dyz", "Dzz"),
}
ATOMIC_NUMBER = {"H": 1.0, "He": 2.0, "Li": 3.0, "Be": 4.0, "B": 5.0, "C": 6.0,
                 "N": 7.0, "O": 8.0, "F": 9.0, "Ne": 10.0}


@dataclass(frozen=True)
class CGF:
    """Contracted Gaussian function: primitives ``(coeff, expo)`` and a label."""
    primitives: Tuple[Tuple[float, float], ...]
    funtype: str

    @property
    def lxyz(self):
        return FUNTYPES[self.funtype]


@dataclass
class AtomData:
    """One atom: coordinates (bohr), its CGFs and its nuclear charge."""
    coord: Tuple[float, float, float]
    basis: List[CGF]
    znumber: float
    label: str = ""


def fac_odd(i: int) -> float:
    """``facOdd`` (IntegralsEvaluation.hs:530-535): (i)!! for odd i, 1 for i < 2."""
    if i % 2 == 0:
        raise ValueError("facOdd needs an odd integer")
    if i < 2:
        return 1.0
    k = (1 + i) // 2
    return math.factorial(2 * k) / (2.0 ** k * math.factorial(k))


def norm_coeff(funtype: str, coefs: Sequence[float], exps: Sequence[float]) -> List[float]:
    """``normCoeff`` (NormalizeBasis.hs:52-59): c / sqrt(ang(e) * (pi/(2e))^1.5)."""
    idx = FUNTYPES[funtype]
    prod = 1.0
    for k in idx:
        prod *= fac_odd(2 * k - 1)
    out = []
    for c, e in zip(coefs, exps):
        ang = prod / (4.0 * e) ** sum(idx)
        out.append(c / math.sqrt(ang * (math.pi / (2.0 * e)) ** 1.5))
    return out


@lru_cache(maxsize=None)
def load_basis_sets():
    path = Path(__file__).with_name("data") / "basis_sets.json"
    return json.loads(path.read_text())["sets"]


def create_cgf(shells) -> List[CGF]:
    """``createCGF`` + ``normGlobal`` for one element's shell list."""
    out: List[CGF] = []
    for sh in shells:
        exps = sh["exps"]
        if sh["kind"] == "SP":
            groups = (("S", sh["coefs"][0]), ("P", sh["coefs"][1]))
        elif sh["kind"] == "S":
            groups = (("S", sh["coefs"][0]),)
        else:
            groups = ((sh["kind"], sh["coefs"][0]),)
        for kind, coefs in groups:
            for lab in SHELL_LABELS[kind]:
                cs = norm_coeff(lab, coefs, exps)
                out.append(CGF(tuple(zip(cs, exps)), lab))
    return out


def basis_for(element: str, basis: str = "sto-3g", variant: str = "text") -> List[CGF]:
    """CGFs of ``element`` in ``basis``.

    ``variant="shipped"`` reproduces the reference's decoded blobs (every SP
    exponent equal to 1.0); ``variant="text"`` keeps the EMSL exponents.
    """
    sets = load_basis_sets()
    key = basis.lower()
    if key not in sets:
        raise KeyError(f"unknown basis set: {basis}")
    return create_cgf(sets[key][variant][element])


def make_atoms(labels: Sequence[str], coords_bohr, basis: str = "sto-3g",
               variant: str = "text") -> List[AtomData]:
    """``createAtomData`` (HsFock/Initialize.hs:38-41) for coordinates in bohr."""
    coords_bohr = np.asarray(coords_bohr, dtype=np.float64).reshape(-1, 3)
    return [AtomData(tuple(float(v) for v in xyz), basis_for(l, basis, variant),
                     ATOMIC_NUMBER[l], l)
            for l, xyz in zip(labels, coords_bohr)]


@dataclass
class FlatBasis:
    """``[AtomData]`` flattened to the structure-of-arrays form of the C ABI."""
    n_atoms: int
    xyz: np.ndarray          # (n_atoms, 3) float64, bohr
    charge: np.ndarray       # (n_atoms,) float64
    n_cgf: int
    cgf_atom: np.ndarray     # (n_cgf,) int32
    cgf_lxyz: np.ndarray     # (n_cgf, 3) int32
    cgf_nprim: np.ndarray    # (n_cgf,) int32
    prim_coef: np.ndarray    # (sum nprim,) float64
    prim_exp: np.ndarray     # (sum nprim,) float64
    labels: List[str] = field(default_factory=list)

    @property
    def n_occupied(self):
        return int(math.floor(float(self.charge.sum()) / 2.0))


def flatten(atoms: Sequence[AtomData]) -> FlatBasis:
    xyz, zs, ca, lx, npr, co, ex = [], [], [], [], [], [], []
    for ia, at in enumerate(atoms):
        xyz.append(at.coord)
        zs.append(at.znumber)
        for cgf in at.basis:
            ca.append(ia)
            lx.append(cgf.lxyz)
            npr.append(len(cgf.primitives))
            for c, e in cgf.primitives:
                co.append(c)
                ex.append(e)
    return FlatBasis(len(atoms), np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3),
                     np.asarray(zs, dtype=np.float64), len(ca),
                     np.asarray(ca, dtype=np.int32), np.asarray(lx, dtype=np.int32).reshape(-1, 3),
                     np.asarray(npr, dtype=np.int32), np.asarray(co, dtype=np.float64),
                     np.asarray(ex, dtype=np.float64), [a.label for a in atoms])


def n_basis(atoms: Sequence[AtomData]) -> int:
    return sum(len(a.basis) for a in atoms)
