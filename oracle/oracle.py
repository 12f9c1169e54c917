"""CPU FP64 oracle: ctypes binding of gbhf_oracle.cpp plus the SCF driver.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()``
(as the checker) and by ``bench.py`` (CPU baseline / reference arm).  The
product library never calls it.

The integral and Fock kernels live in C++ (gbhf_oracle.cpp).  The SCF driver
below restates, step by step, the reference's Haskell driver:

* ``scf_hf``            HartreeFock/HartreeFock.hs:70-87
* ``scf_diis`` loop     HartreeFock/HartreeFock.hs:104-123
* ``harris_functional`` HartreeFock/HartreeFock.hs:128-149
* ``calc_density``      HartreeFock/HartreeFock.hs:195-208
* ``diagonal_hf``       HartreeFock/HartreeFock.hs:263-273
* ``variational_e``     HartreeFock/HartreeFock.hs:277-287
* ``nuclear_rep``       HartreeFock/HartreeFock.hs:300-305
* ``sad_density``       no reference counterpart: the superposition-of-atomic-
                         densities guess of the library (restated for checking)
* ``calc_error_mtx``, ``diis_driver``, ``diis``, ``update_diis``
                         HartreeFock/DIIS.hs:55-140
* ``gauss_elem``        NumericalTools/GaussElimination.hs:42-98
* ``symm_ortho``        HartreeFock/BasisOrthogonalization.hs:26-34
* ``eigen_solve``       NumericalTools/EigenValues.hs:29-31 (LAPACK through
                         numpy, as the reference goes through hmatrix/LAPACK),
                         ascending sort as VectorTools.hs:27-31.

Parity status: the reference cannot run here (no GHC toolchain), so this
oracle is pinned only by the known-answer data the reference carries (the
Boys-function table in Boys.hs:27-39, the Gauss-elimination system in
GaussElimination.hs:115-119) and by textbook energies of the reference's own
sample projects; see tests/test_oracle_*.py.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
SRC = HERE / "gbhf_oracle.cpp"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(force=False):
    """Compile the oracle with g++ (OpenMP) into oracle/_build/liboracle.so."""
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB_PATH
    LIB_PATH.parent.mkdir(exist_ok=True)
    tmp = LIB_PATH.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.check_call(["g++", "-O2", "-fopenmp", "-shared", "-fPIC", "-std=c++17",
                           "-o", str(tmp), str(SRC)])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        L.orc_boys_exact.restype = C.c_double
        L.orc_boys_exact.argtypes = [C.c_int, C.c_double]
        L.orc_boys_ref.restype = C.c_double
        L.orc_boys_ref.argtypes = [C.c_double, C.c_double]
        L.orc_asympt_boys_ref.restype = C.c_double
        L.orc_asympt_boys_ref.argtypes = [C.c_double, C.c_double]
        L.orc_boys_taylor.restype = C.c_double
        L.orc_boys_taylor.argtypes = [_dp, C.c_int, C.c_double]
        L.orc_boys_exact_vec.argtypes = [C.c_int, C.c_double, _dp]
        L.orc_boys_ref_grid.argtypes = [_dp]
        L.orc_gauss_legendre.argtypes = [C.c_int, _dp, _dp]
        L.orc_basis_create.restype = C.c_void_p
        L.orc_basis_create.argtypes = [C.c_int, _dp, _dp, C.c_int, _ip, _ip, _ip, _dp, _dp, _dp]
        L.orc_basis_destroy.argtypes = [C.c_void_p]
        L.orc_nshells.argtypes = [C.c_void_p]
        L.orc_shell_info.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip, _ip]
        L.orc_overlap.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_kinetic.argtypes = [C.c_void_p, _dp]
        L.orc_hcore.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_eri_canonical_len.restype = C.c_long
        L.orc_eri_canonical_len.argtypes = [C.c_int]
        L.orc_eri_canonical.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_canonical_index.restype = C.c_long
        L.orc_canonical_index.argtypes = [C.c_int] * 5
        L.orc_eri.restype = C.c_double
        L.orc_eri.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_fock_canonical.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        L.orc_fock_direct.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, _dp, C.POINTER(C.c_longlong)]
        L.orc_shell_pair_bounds.argtypes = [C.c_void_p, _dp]
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def _pi(a):
    return a.ctypes.data_as(_ip)


# ------------------------------------------------------------------ Boys ----

def boys_exact(m, x):
    return lib().orc_boys_exact(int(m), float(x))


def boys_ref(m, x):
    """The reference's ``boysF m x`` (quadrature / erf / asymptotic)."""
    return lib().orc_boys_ref(float(m), float(x))


_GRID = None


def boys_ref_grid():
    """``generateGridBoys 0.1``: array (15, 1001), grid[m, i] = boysF m (0.1 i)."""
    global _GRID
    if _GRID is None:
        g = np.zeros(15 * 1001)
        lib().orc_boys_ref_grid(_p(g))
        _GRID = g
    return _GRID.reshape(15, 1001)


def boys_taylor(m, x, grid=None):
    g = np.ascontiguousarray(boys_ref_grid() if grid is None else grid, dtype=np.float64).ravel()
    return lib().orc_boys_taylor(_p(g), int(m), float(x))


def gauss_legendre(n):
    x = np.zeros(n // 2)
    w = np.zeros(n // 2)
    lib().orc_gauss_legendre(n, _p(x), _p(w))
    return x, w


# ----------------------------------------------------------------- basis ----

class OracleBasis:
    """Owns an oracle basis handle built from a ``gbhf.basis.FlatBasis``."""

    def __init__(self, fb, grid=None):
        self.fb = fb
        self.n = int(fb.n_cgf)
        self._keep = [np.ascontiguousarray(a) for a in (
            fb.xyz.ravel(), fb.charge, fb.cgf_atom, fb.cgf_lxyz.ravel(), fb.cgf_nprim,
            fb.prim_coef, fb.prim_exp)]
        self.grid = np.ascontiguousarray(boys_ref_grid() if grid is None else grid).ravel()
        k = self._keep
        self.h = lib().orc_basis_create(int(fb.n_atoms), _p(k[0]), _p(k[1]), self.n, _pi(k[2]),
                                        _pi(k[3]), _pi(k[4]), _p(k[5]), _p(k[6]), _p(self.grid))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_basis_destroy(self.h)
            self.h = None

    @property
    def ntri(self):
        return self.n * (self.n + 1) // 2

    def shells(self):
        ns = lib().orc_nshells(self.h)
        arrs = [np.zeros(ns, dtype=np.int32) for _ in range(5)]
        lib().orc_shell_info(self.h, *[_pi(a) for a in arrs])
        return dict(zip(("atom", "L", "ncomp", "nprim", "first_fn"), arrs))

    def overlap(self, ref_compat=True):
        out = np.zeros(self.ntri)
        lib().orc_overlap(self.h, int(ref_compat), _p(out))
        return out

    def kinetic(self):
        out = np.zeros(self.ntri)
        lib().orc_kinetic(self.h, _p(out))
        return out

    def hcore(self, ref_compat=True):
        out = np.zeros(self.ntri)
        lib().orc_hcore(self.h, int(ref_compat), _p(out))
        return out

    def eri_canonical(self, ref_compat=True):
        out = np.zeros(lib().orc_eri_canonical_len(self.n))
        lib().orc_eri_canonical(self.h, int(ref_compat), _p(out))
        return out

    def eri(self, i, j, k, l, ref_compat=True):
        return lib().orc_eri(self.h, int(ref_compat), i, j, k, l)

    def fock_direct(self, H, D, schwarz=1e-12, density_screen=True):
        """H + G(D) by shell quartets; drops Q_AB Q_CD < schwarz and (density_screen)
        Q_AB Q_CD max|D| over the quartet's six density blocks < schwarz, as the device build."""
        F = np.zeros(self.ntri)
        st = np.zeros(3, dtype=np.int64)
        lib().orc_fock_direct(self.h, _p(np.ascontiguousarray(H)), _p(np.ascontiguousarray(D)),
                              float(schwarz), int(bool(density_screen)), _p(F),
                              st.ctypes.data_as(C.POINTER(C.c_longlong)))
        return F, st

    def shell_pair_bounds(self):
        ns = lib().orc_nshells(self.h)
        q = np.zeros(ns * (ns + 1) // 2)
        lib().orc_shell_pair_bounds(self.h, _p(q))
        return q


def fock_canonical(H, D, eri):
    n = dim_triang(len(H))
    F = np.zeros_like(H)
    lib().orc_fock_canonical(n, _p(np.ascontiguousarray(H)), _p(np.ascontiguousarray(D)),
                             _p(np.ascontiguousarray(eri)), _p(F))
    return F


def canonical_index(n, i, j, k, l):
    return lib().orc_canonical_index(n, i, j, k, l)


# --------------------------------------------------------- flat layouts ----

def dim_triang(a):
    """``dimTriang`` (LinearAlgebra.hs:314-316)."""
    p = int(math.floor(math.sqrt(1 + 8 * a)))
    return (p - 1) // 2


def index_dim2_to_flat(dim, x, y):
    """``indexDIM2toFlat`` (LinearAlgebra.hs:250-253), literal form."""
    def calc_elem(w):
        if w == 0:
            return 0
        return sum(dim - s for s in range(max(w, 0)))
    return calc_elem(x) + (y - x) if x <= y else calc_elem(y) + (x - y)


def index_flat_to_dim2(dim, i):
    """``indexFlat2DIM2`` (LinearAlgebra.hs:240-246), literal form."""
    x, n = i, 0
    while not x < dim - n:
        x -= dim - n
        n += 1
    calc = 0 if n == 0 else sum(dim - s for s in range(n))
    return n, i + n - calc


def tri_to_square(flat):
    n = dim_triang(len(flat))
    iu = np.triu_indices(n)
    m = np.zeros((n, n))
    m[iu] = flat
    m[(iu[1], iu[0])] = flat
    return m


def square_to_tri(m):
    return np.asarray(m)[np.triu_indices(m.shape[0])].copy()


def sort_keys(k):
    """``sortKeys`` (HartreeFock.hs:153-156)."""
    i, j, kk, l = k
    l1, l2 = sorted([i, j]), sorted([kk, l])
    return l1 + l2 if l1 <= l2 else l2 + l1


def _sum_index_triang(n):
    return (n * n + n) // 2


def _sum_first_index(n):
    return n + _sum_index_triang(n - 1) + sum(_sum_index_triang(n) - k for k in range(1, n))


def _total_first_index(n, first):
    return sum(_sum_first_index(n - m) for m in range(first))


def _select_position(n, key):
    i, j, k, l = key
    if i == j == k:
        return l - i
    if i == j:
        ip = lambda x: x - (i + 1)
        return (n - i) + index_dim2_to_flat(ip(n), ip(k), ip(l))
    return ((n - i) + _sum_index_triang(n - 1 - i)
            + sum(_sum_index_triang(n - i) - m for m in range(1, j - i))
            + (index_dim2_to_flat(n, k, l) - index_dim2_to_flat(n, i, j)))


def four_index_to_flat(n, key):
    """``fourIndex2Flat`` (LinearAlgebra.hs:266-283), literal form (any n)."""
    return _total_first_index(n, key[0]) + _select_position(n, key)


# ----------------------------------------------------- dense linear algebra ----

def eigen_solve(m):
    """``eigenSolve``: LAPACK eigenpairs, eigenvalues ascending, vectors in columns."""
    w, v = np.linalg.eigh(m)
    order = np.argsort(w, kind="mergesort")
    return w[order], v[:, order]


def symm_ortho(s_sq):
    w, u = eigen_solve(s_sq)
    return (u * (1.0 / np.sqrt(w))) @ u.T


def calc_density(coeff, occupied):
    c = coeff[:, :occupied]
    return square_to_tri(2.0 * c @ c.T)


def diagonal_hf(fock_flat, x, occupied):
    f = x.T @ tri_to_square(fock_flat) @ x
    eps, cp = eigen_solve(f)
    c = x @ cp
    return c, calc_density(c, occupied), eps


def variational_e(core, fock, density):
    return 0.5 * float(np.sum(tri_to_square(density) * (tri_to_square(core) + tri_to_square(fock))))


def nuclear_rep(xyz, z):
    e = 0.0
    for a in range(len(z)):
        for b in range(a + 1, len(z)):
            e += z[a] * z[b] / float(np.linalg.norm(xyz[a] - xyz[b]))
    return e


def calc_error_mtx(f, s, d, x):
    F, S, D = tri_to_square(f), tri_to_square(s), tri_to_square(d)
    e = F @ (D @ S) - (S @ D) @ F
    return x.T @ (e @ x)


def gauss_elem(mtx, vec):
    """Unpivoted Gauss elimination with the reference's failure rules.

    Returns None when a row of the eliminated matrix has no entry with
    magnitude above 1e-6 or when it holds NaN/Inf (GaussElimination.hs:71-88).
    """
    a = np.array(mtx, dtype=np.float64)
    b = np.array(vec, dtype=np.float64)
    n = a.shape[0]
    with np.errstate(all="ignore"):
        for k in range(n):
            old = a.copy()
            for i in range(k + 1, n):
                alpha = old[i, k] / old[k, k]
                a[i, k:] = old[i, k:] - alpha * old[k, k:]
                b[i] = b[i] - alpha * b[k]
        if not np.all(np.any(np.abs(a) > 1e-6, axis=1)) or not np.all(np.isfinite(a)):
            return None
        x = np.zeros(n)
        for k in range(n - 1, -1, -1):
            x[k] = (b[k] - np.dot(x[k + 1:], a[k, k + 1:])) * (1.0 / a[k, k])
    return x


@dataclass
class DataDIIS:
    errors: List[np.ndarray] = field(default_factory=list)   # newest first
    focks: List[np.ndarray] = field(default_factory=list)
    size: int = 5


def update_diis(dat, e, f):
    es, fs = [e] + dat.errors, [f] + dat.focks
    if len(es) >= dat.size:
        es, fs = es[:-1], fs[:-1]
    return DataDIIS(es, fs, dat.size)


def diis(e, f, dat):
    while True:
        fs = [f] + dat.focks
        es = [e] + dat.errors
        dim1 = len(fs)
        b = np.zeros((dim1 + 1, dim1 + 1))
        for i in range(dim1):
            for j in range(dim1):
                b[i, j] = np.trace(es[i].T @ es[j])
        b[dim1, :dim1] = -1
        b[:dim1, dim1] = -1
        rhs = np.zeros(dim1 + 1)
        rhs[-1] = -1
        cs = gauss_elem(b, rhs)
        if cs is None:
            dat = DataDIIS(dat.errors[:-1], dat.focks[:-1], dat.size)
            continue
        return sum(cs[k] * fs[k] for k in range(dim1)), dat


def diis_driver(e, f, dat, step, switch_on, start_threshold=0.1):
    if not switch_on:
        if step > 0 and np.max(np.abs(e)) < start_threshold:
            return f, update_diis(dat, e, f), True
        return f, dat, False
    new_f, cur = diis(e, f, dat)
    return new_f, update_diis(cur, e, f), True


def harris_guess_terms(eri, n_tri, occupied):
    """``computeGuessIntegrals`` (HartreeFock.hs:138-149) with its index semantics.

    The reference calls ``indexFlat2DIM2 dim`` with dim = the flat length, so
    (i, j) = (0, idx), and ``fourIndex2Flat occupied``.  Raises IndexError where
    the reference's bounds-checked lookup fails.
    """
    out = np.zeros(n_tri)
    for idx in range(n_tri):
        s = 0.0
        for k in range(occupied):
            f1 = four_index_to_flat(occupied, sort_keys([0, idx, k, k]))
            f2 = four_index_to_flat(occupied, sort_keys([0, k, k, idx]))
            if not (0 <= f1 < len(eri) and 0 <= f2 < len(eri)):
                raise IndexError("Harris guess reads ERI index %d/%d outside [0,%d)" % (f1, f2, len(eri)))
            s += eri[f1] - 0.5 * eri[f2]
        out[idx] = 2.0 * s
    return out


# -------------------------------------------------------------- SCF driver ----

def _atom_sub_basis(fb, a):
    """Functions of atom ``a`` as a one-atom basis at the origin, with their indices."""
    idx = np.where(fb.cgf_atom == a)[0]
    off = np.concatenate([[0], np.cumsum(fb.cgf_nprim)])
    coef = np.concatenate([fb.prim_coef[off[i]:off[i + 1]] for i in idx])
    expo = np.concatenate([fb.prim_exp[off[i]:off[i + 1]] for i in idx])
    sub = type(fb)(1, np.zeros((1, 3)), fb.charge[a:a + 1].astype(np.float64), len(idx),
                   np.zeros(len(idx), np.int32), np.ascontiguousarray(fb.cgf_lxyz[idx], dtype=np.int32),
                   np.ascontiguousarray(fb.cgf_nprim[idx], dtype=np.int32), coef, expo)
    return sub, idx


def fractional_occupations(eps, nel, tol=1e-5):
    """Aufbau with 2 electrons per orbital; a partly filled set of orbitals
    whose energies agree to ``tol`` shares its electrons equally."""
    occ = np.zeros(len(eps))
    left, i = float(nel), 0
    while left > 1e-12 and i < len(eps):
        j = i
        while j + 1 < len(eps) and abs(eps[j + 1] - eps[i]) < tol:
            j += 1
        take = min(left, 2.0 * (j - i + 1))
        occ[i:j + 1] = take / (j - i + 1)
        left -= take
        i = j + 1
    return occ


def atomic_density(fb1, max_iter=200):
    """Spherically averaged fractional-occupation RHF density of one neutral
    atom (square, in its own functions): Roothaan steps from the core
    Hamiltonian, the first four averaged with the previous density, until
    max|dD| < 1e-10."""
    ob = OracleBasis(fb1)
    h, s, eri = ob.hcore(False), ob.overlap(False), ob.eri_canonical(False)
    x = symm_ortho(tri_to_square(s))
    nel = float(fb1.charge.sum())
    f, d = tri_to_square(h), None
    for it in range(max_iter):
        eps, cp = np.linalg.eigh(x.T @ f @ x)
        c = x @ cp
        dn = (c * fractional_occupations(eps, nel)) @ c.T
        change = 1.0 if d is None else float(np.max(np.abs(dn - d)))
        d = dn if (d is None or it >= 4) else 0.5 * (dn + d)
        if change < 1e-10:
            break
        f = tri_to_square(fock_canonical(h, square_to_tri(d), eri))
    return d


def sad_density(fb):
    """Superposition of atomic densities (flat upper triangle): block-diagonal
    assembly of ``atomic_density`` for every atom, computed once per distinct
    atom (charge and functions)."""
    n = int(fb.n_cgf)
    dens = np.zeros((n, n))
    cache = {}
    for a in range(int(fb.n_atoms)):
        sub, idx = _atom_sub_basis(fb, a)
        key = (float(sub.charge[0]), sub.cgf_lxyz.tobytes(), sub.cgf_nprim.tobytes(), sub.prim_coef.tobytes(),
               sub.prim_exp.tobytes())
        if key not in cache:
            cache[key] = atomic_density(sub)
        dens[np.ix_(idx, idx)] = cache[key]
    return square_to_tri(dens)


@dataclass
class SCFOptions:
    ref_compat: bool = True        # reference numerics + reference driver rules
    guess: str = "harris"          # "harris" | "core" | "sad" | "density"
    diis_size: int = 5             # vectors in the extrapolation (current + stored)
    max_iter: int = 30
    conv_error: float = 1e-7       # max|e| (reference rule, used when ref_compat)
    conv_energy: float = 1e-10     # |dE| (baseline rule)
    conv_density: float = 1e-8     # RMS dD (baseline rule)
    diis_start: float = 0.1
    schwarz: float = 1e-12
    charge: float = 0.0
    direct: bool = False           # shell-based direct Fock instead of stored ERIs
    stop_rule: str = ""            # "reference" | "energy"; default follows ref_compat
    guess_density: Optional[np.ndarray] = None   # flat start density for guess="density" (restart)

    @staticmethod
    def reference():
        return SCFOptions()

    @staticmethod
    def baseline(**kw):
        o = SCFOptions(ref_compat=False, guess="core", diis_size=6, diis_start=1e30, direct=True)
        for k, v in kw.items():
            setattr(o, k, v)
        return o


@dataclass
class SCFResult:
    energy: float
    fock: np.ndarray
    coeff: np.ndarray
    density: np.ndarray
    orb_energies: np.ndarray
    iterations: int
    energies: List[float]
    converged: bool


class SCFNotConverged(RuntimeError):
    pass


def scf(fb, opts: Optional[SCFOptions] = None, grid=None):
    """Closed-shell RHF of a ``FlatBasis`` following ``scfHF``/``scfDIIS``."""
    for item in scf_steps(fb, opts, grid):
        if item is not None and item[1] is not None:
            return item[1]
    raise SCFNotConverged("SCF maxium steps exceeded")   # scf_steps raises first


def scf_steps(fb, opts: Optional[SCFOptions] = None, grid=None):
    """The driver of ``scf``, one SCF iteration at a time: yields ``None``
    after the setup (integrals, orthogonaliser, start density), then
    ``(step, result)`` after every iteration, ``result`` being the
    ``SCFResult`` at convergence and ``None`` before; raises
    ``SCFNotConverged`` after ``max_iter`` steps (HartreeFock.hs:123)."""
    opts = opts or SCFOptions.reference()
    ob = OracleBasis(fb, grid)
    ref = opts.ref_compat
    ref_stop = (opts.stop_rule or ("reference" if ref else "energy")) == "reference"
    occupied = int(math.floor((float(fb.charge.sum()) - opts.charge) / 2.0))
    e_nn = nuclear_rep(fb.xyz, fb.charge)
    core = ob.hcore(ref)
    s = ob.overlap(ref)
    x = symm_ortho(tri_to_square(s))
    eri = None
    if not opts.direct:
        eri = ob.eri_canonical(ref)

    def fock(d):
        if opts.direct:
            return ob.fock_direct(core, d, opts.schwarz)[0]
        return fock_canonical(core, d, eri)

    if opts.guess == "harris":
        if eri is None:
            eri = ob.eri_canonical(ref)
        g = harris_guess_terms(eri, len(core), occupied)
        _, density, _ = diagonal_hf(core + g, x, occupied)
    elif opts.guess == "sad":
        density = sad_density(fb)
    elif opts.guess == "density":
        density = np.array(opts.guess_density, dtype=np.float64, copy=True)
        if density.shape != core.shape:
            raise ValueError("guess density does not match the basis")
    else:
        _, density, _ = diagonal_hf(core, x, occupied)
    yield None
    dat = DataDIIS(size=opts.diis_size)
    switch = False
    energies = []
    e_prev = None
    for step in range(opts.max_iter):
        f = fock(density)
        err = calc_error_mtx(f, s, density, x)
        f_diis, dat, switch = diis_driver(err, f, dat, step, switch, opts.diis_start)
        c, new_density, eps = diagonal_hf(f_diis, x, occupied)
        if ref_stop:
            etot = variational_e(core, f_diis, new_density) + e_nn
            energies.append(etot)
            if step != 0 and np.max(np.abs(err)) < opts.conv_error:
                yield step, SCFResult(etot, f_diis, c, new_density, eps, step + 1, energies, True)
                return
        else:
            etot = variational_e(core, f, density) + e_nn
            energies.append(etot)
            rms = float(np.sqrt(np.mean((tri_to_square(new_density) - tri_to_square(density)) ** 2)))
            if e_prev is not None and abs(etot - e_prev) < opts.conv_energy and rms < opts.conv_density:
                yield step, SCFResult(etot, f, c, new_density, eps, step + 1, energies, True)
                return
            e_prev = etot
        density = new_density
        yield step, None
    raise SCFNotConverged("SCF maxium steps exceeded")


# ------------------------------------------------------------ open shell ----

def eri_tensor(ob, n):
    """Full (ab|cd) tensor from the oracle's contracted ERIs (exact numerics), small n."""
    t = np.zeros((n, n, n, n))
    for i in range(n):
        for j in range(i + 1):
            for k in range(n):
                for l in range(k + 1):
                    if k * (k + 1) // 2 + l > i * (i + 1) // 2 + j:
                        continue
                    v = ob.eri(i, j, k, l, ref_compat=False)
                    for (a, b, c, d) in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                                         (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                        t[a, b, c, d] = v
    return t


@dataclass
class UHFResult:
    energy: float
    density_alpha: np.ndarray   # square
    density_beta: np.ndarray
    n_alpha: int
    n_beta: int
    s2: float
    iterations: int


def uhf(fb, multiplicity, charge=0.0, max_iter=200, conv_energy=1e-12, conv_density=1e-10, diis_size=6):
    """Unrestricted HF with a core-Hamiltonian start and DIIS over both spins
    (the reference has no open-shell SCF; this is the textbook UHF of Pople and
    Nesbet, F_a = H + J(D_a + D_b) - K(D_a)), in numpy on the full ERI tensor."""
    ob = OracleBasis(fb)
    n = fb.n_cgf
    S = tri_to_square(ob.overlap(False))
    H = tri_to_square(ob.hcore(False))
    w, U = np.linalg.eigh(S)
    X = (U / np.sqrt(w)) @ U.T
    nel = int(round(float(fb.charge.sum()) - charge))
    na = (nel + multiplicity - 1) // 2
    nb = nel - na
    eri = eri_tensor(ob, n)
    e_nn = nuclear_rep(fb.xyz, fb.charge)

    def dens(F, nocc):
        e, V = np.linalg.eigh(X.T @ F @ X)
        C = X @ V
        return C[:, :nocc] @ C[:, :nocc].T

    Da, Db = dens(H, na), dens(H, nb)
    hist = []
    e_prev = None
    for it in range(max_iter):
        J = np.einsum("abcd,cd->ab", eri, Da + Db)
        Fa = H + J - np.einsum("acbd,cd->ab", eri, Da)
        Fb = H + J - np.einsum("acbd,cd->ab", eri, Db)
        energy = 0.5 * (np.sum((Da + Db) * H) + np.sum(Da * Fa) + np.sum(Db * Fb)) + e_nn
        ea = X.T @ (Fa @ Da @ S - S @ Da @ Fa) @ X
        eb = X.T @ (Fb @ Db @ S - S @ Db @ Fb) @ X
        hist.insert(0, (ea, eb, Fa, Fb))
        del hist[diis_size:]
        fa, fb_ = Fa, Fb
        while it > 0 and len(hist) >= 2:
            k = len(hist)
            B = -np.ones((k + 1, k + 1))
            B[k, k] = 0
            for i in range(k):
                for j in range(k):
                    B[i, j] = np.sum(hist[i][0] * hist[j][0]) + np.sum(hist[i][1] * hist[j][1])
            rhs = np.zeros(k + 1)
            rhs[k] = -1
            try:
                x = np.linalg.solve(B, rhs)[:k]
            except np.linalg.LinAlgError:
                hist.pop()
                continue
            fa = sum(x[i] * hist[i][2] for i in range(k))
            fb_ = sum(x[i] * hist[i][3] for i in range(k))
            break
        Na, Nb = dens(fa, na), dens(fb_, nb)
        rms = math.sqrt((np.sum((Na - Da) ** 2) + np.sum((Nb - Db) ** 2)) / (2.0 * n * n))
        if e_prev is not None and abs(energy - e_prev) < conv_energy and rms < conv_density:
            sz = 0.5 * (na - nb)
            s2 = sz * (sz + 1) + nb - np.sum((S @ Na @ S) * Nb)
            return UHFResult(energy, Na, Nb, na, nb, float(s2), it + 1)
        e_prev = energy
        Da, Db = Na, Nb
    raise SCFNotConverged("UHF did not converge")
