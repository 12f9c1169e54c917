"""Host-side mirror of the reference's ``Science.QuantumChemistry`` call surface.

Same names (snake_case), argument meaning and error behaviour as the Haskell
functions, every one running on the GPU through libgbhf:

======================  =====================================================
this module             reference
======================  =====================================================
generate_grid_boys      NumericalTools/TableBoys.hs:58-63 generateGridBoys
boys_taylor             NumericalTools/TableBoys.hs:45-51 boysTaylor
mtx_overlap             Integrals/IntegralsEvaluation.hs:169-177 mtxOverlap
hcore                   Integrals/IntegralsEvaluation.hs:227-240 hcore
calc_integrals          HartreeFock/HartreeFock.hs:166-181 calcIntegrals
fock                    HartreeFock/HartreeFock.hs:213-222 fock
symm_ortho              HartreeFock/BasisOrthogonalization.hs:26-34 symmOrtho
eigen_solve             NumericalTools/EigenValues.hs:29-31 eigenSolve
diagonal_hf             HartreeFock/HartreeFock.hs:263-273 diagonalHF
calc_error_mtx          HartreeFock/DIIS.hs:119-132 calcErrorMtx
diis, diis_driver       HartreeFock/DIIS.hs:55-88
gauss_elem              NumericalTools/GaussElimination.hs:42-46 gaussElem
scf_hf                  HartreeFock/HartreeFock.hs:70-87 scfHF
======================  =====================================================

Arrays follow the reference layouts: symmetric matrices as the flat upper
triangle (numpy 1-D), square matrices as (N, N) numpy arrays.  Errors raise
``gbhf.GBHFError``; a non-converged SCF raises ``NotConverged`` (the
reference's ``error "SCF maxium steps exceeded"``) and a singular Gauss
elimination returns ``None`` (the reference's ``Nothing``).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import _lib
from .basis import AtomData, flatten

_ctx: Optional[_lib.Context] = None
_ctx_key = None


def context() -> _lib.Context:
    global _ctx
    if _ctx is None:
        _ctx = _lib.Context(0)
    return _ctx


def _bind(atoms: Sequence[AtomData]) -> _lib.Context:
    global _ctx_key
    ctx = context()
    key = tuple((a.coord, tuple(a.basis), a.znumber) for a in atoms)
    if key != _ctx_key:
        ctx.set_basis(flatten(atoms))
        _ctx_key = key
    return ctx


@dataclass
class HFData:
    """``HFData`` (GlobalTypes.hs:122-128)."""
    fock: np.ndarray
    coeff: np.ndarray
    density: np.ndarray
    orb_energies: np.ndarray
    energy: float
    iterations: int = 0


@dataclass
class DataDIIS:
    """``DataDIIS`` (HartreeFock/DIIS.hs:51): stored error matrices and Fock
    matrices, newest first, and the DIIS size."""
    errors: List[np.ndarray] = field(default_factory=list)
    focks: List[np.ndarray] = field(default_factory=list)
    size: int = 5


def generate_grid_boys(delta: float = 0.1) -> np.ndarray:
    """The (15, 1001) table boysF m (0.1 i), computed on the device."""
    if delta != 0.1:
        raise ValueError("the reference grid is defined for delta = 0.1")
    return context().generate_boys_grid()


def boys_taylor(grid: np.ndarray, m: int, x) -> np.ndarray:
    ctx = context()
    ctx.set_boys_grid(grid)
    return ctx.boys(_lib.MODE_REFERENCE, int(m), np.atleast_1d(x))[:, int(m)]


def mtx_overlap(atoms, mode=_lib.MODE_REFERENCE) -> np.ndarray:
    return _bind(atoms).overlap(mode)


def hcore(grid_boys, atoms, mode=_lib.MODE_REFERENCE) -> np.ndarray:
    ctx = _bind(atoms)
    if grid_boys is not None:
        ctx.set_boys_grid(grid_boys)
    return ctx.hcore(mode)


def calc_integrals(grid_boys, atoms, mode=_lib.MODE_REFERENCE) -> np.ndarray:
    ctx = _bind(atoms)
    if grid_boys is not None:
        ctx.set_boys_grid(grid_boys)
    return ctx.eri_canonical(mode)


def fock(atoms, core, density, integrals=None, mode=None, precision=_lib.PREC_FP64, schwarz=1e-12,
         mixed=1e-4) -> np.ndarray:
    """F = H + G(D).  With stored ``integrals`` (reference mode) the canonical
    array is contracted on the device as calcGmatrix does; without them the
    direct J/K kernels recompute the integrals."""
    ctx = _bind(atoms)
    if mode is None:
        mode = _lib.MODE_REFERENCE if integrals is not None else _lib.MODE_EXACT
    return ctx.fock(core, density, mode, precision, schwarz, mixed)


def symm_ortho(s_square) -> np.ndarray:
    return context().symm_ortho(s_square)


def eigen_solve(a_square):
    return context().eigen_solve(a_square)


def diagonal_hf(fock_flat, xmatrix, occupied):
    c, d, e = context().diagonal_hf(fock_flat, xmatrix, occupied)
    return c, d, e


def calc_error_mtx(f, s, d, xmatrix) -> np.ndarray:
    return context().diis_error(f, s, d, xmatrix)


def gauss_elem(mtx, vec):
    try:
        return context().gauss_elem(mtx, vec)
    except _lib.GBHFError as e:
        if e.status == 3:
            return None
        raise


def _update_diis(dat: DataDIIS, e, f) -> DataDIIS:
    es, fs = [e] + dat.errors, [f] + dat.focks
    if len(es) >= dat.size:
        es, fs = es[:-1], fs[:-1]
    return DataDIIS(es, fs, dat.size)


def diis(e, f, dat: DataDIIS):
    """Extrapolated Fock matrix and the (possibly trimmed) history."""
    new_f, used = context().diis_extrapolate([e] + dat.errors, [f] + dat.focks)
    return new_f, DataDIIS(dat.errors[:used], dat.focks[:used], dat.size)


def diis_driver(e, f, dat: DataDIIS, step: int, switch_on: bool):
    if not switch_on:
        if step > 0 and np.max(np.abs(e)) < 0.1:
            return f, _update_diis(dat, e, f), True
        return f, dat, False
    new_f, cur = diis(e, f, dat)
    return new_f, _update_diis(cur, e, f), True


def scf_hf(atoms, charge: float = 0.0, logger: Optional[Callable[[str], None]] = None,
           opts: Optional[_lib.SCFOpts] = None) -> HFData:
    """Closed-shell RHF; by default the reference's driver and numerics
    (Harris guess, DIIS-5, stop on max|e| < 1e-7, at most 30 steps)."""
    ctx = _bind(atoms)
    if opts is None:
        opts = _lib.reference_opts()
    opts.charge = float(charge)
    if opts.mode == _lib.MODE_REFERENCE:
        ctx.generate_boys_grid()
    r = ctx.scf(opts)
    if logger:
        logger("total Energy: %.8f\n" % r["energy"])
    return HFData(r["fock"], r["coeff"], r["density"], r["orb_energies"], r["energy"], r["iterations"])
