"""ctypes binding of libgbhf (include/gbhf.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly when ``gbhf/_build/libgbhf.so`` is missing, and ``Context``
raises when no GPU is available.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libgbhf.so"
HEADER = Path(__file__).resolve().parents[2] / "include" / "gbhf.h"

STATUS = {0: "GBHF_OK", 1: "GBHF_ERR_BAD_INPUT", 2: "GBHF_ERR_NOT_CONVERGED", 3: "GBHF_ERR_SINGULAR",
          4: "GBHF_ERR_CUDA", 5: "GBHF_ERR_DEVICE_TIMEOUT", 6: "GBHF_ERR_NO_DEVICE", 7: "GBHF_ERR_UNSUPPORTED",
          8: "GBHF_ERR_INDEX"}
MODE_REFERENCE, MODE_EXACT = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
GUESS_HARRIS, GUESS_CORE, GUESS_SAD, GUESS_DENSITY = 0, 1, 2, 3

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p


class GBHFError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status
        self.name = STATUS.get(status, str(status))


class NotConverged(GBHFError):
    """Mirrors the reference's ``error "SCF maxium steps exceeded"``."""


class SCFOpts(C.Structure):
    _fields_ = [("mode", C.c_int), ("precision", C.c_int), ("guess", C.c_int), ("diis_size", C.c_int),
                ("max_iter", C.c_int), ("incremental", C.c_int), ("full_rebuild_every", C.c_int),
                ("final_fp64", C.c_int), ("ref_stop_rule", C.c_int), ("conv_error", C.c_double),
                ("conv_energy", C.c_double), ("conv_density", C.c_double), ("diis_start", C.c_double),
                ("schwarz_cutoff", C.c_double), ("mixed_cutoff", C.c_double), ("charge", C.c_double),
                ("grad_mixed_cutoff", C.c_double), ("autotune", C.c_int)]


class UHFResultC(C.Structure):
    _fields_ = [("energy", C.c_double), ("iterations", C.c_int), ("converged", C.c_int), ("n_alpha", C.c_int),
                ("n_beta", C.c_int), ("s2", C.c_double), ("density_alpha_flat", _dp), ("density_beta_flat", _dp),
                ("orb_energies_alpha", _dp), ("orb_energies_beta", _dp)]


class SCFResultC(C.Structure):
    _fields_ = [("energy", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("n_occupied", C.c_int), ("nuclear_repulsion", C.c_double), ("fock_flat", _dp),
                ("coeff", _dp), ("density_flat", _dp), ("orb_energies", _dp), ("eri_quartets", C.c_double),
                ("eri_fn_quartets", C.c_double), ("eri_prim_quartets", C.c_double),
                ("eri_fp32_fraction", C.c_double), ("fock_builds", C.c_double)]


_lib = None


def load():
    """Load libgbhf.so (built by ``gbhf.build``); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"libgbhf.so not built ({LIB_PATH}); run __graft_entry__.build() or "
                          "python -m gbhf.build")
    L = C.CDLL(str(LIB_PATH))
    st = C.c_int
    sigs = {
        "gbhf_version": (C.c_int, []),
        "gbhf_create": (st, [C.POINTER(_vp), C.c_int]),
        "gbhf_destroy": (st, [_vp]),
        "gbhf_last_error": (C.c_char_p, [_vp]),
        "gbhf_set_basis": (st, [_vp, C.c_int, _dp, _dp, C.c_int, _ip, _ip, _ip, _dp, _dp]),
        "gbhf_set_boys_grid": (st, [_vp, _dp]),
        "gbhf_generate_boys_grid": (st, [_vp, _dp]),
        "gbhf_boys": (st, [_vp, C.c_int, C.c_int, C.c_int, _dp, _dp]),
        "gbhf_overlap": (st, [_vp, C.c_int, _dp]),
        "gbhf_hcore": (st, [_vp, C.c_int, _dp]),
        "gbhf_eri_canonical_length": (C.c_int64, [C.c_int]),
        "gbhf_eri_canonical": (st, [_vp, C.c_int, _dp, C.c_int64]),
        "gbhf_fock": (st, [_vp, C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp]),
        "gbhf_symm_ortho": (st, [_vp, C.c_int, _dp, _dp]),
        "gbhf_eigen_solve": (st, [_vp, C.c_int, _dp, _dp, _dp]),
        "gbhf_eigen_solve_noalloc": (st, [C.c_int, _vp, _vp, _vp, _vp]),
        "gbhf_diagonal_hf": (st, [_vp, C.c_int, _dp, _dp, C.c_int, _dp, _dp, _dp]),
        "gbhf_sad_density": (st, [_vp, _dp]),
        "gbhf_set_guess_density": (st, [_vp, _dp]),
        "gbhf_scf_uhf": (st, [_vp, C.POINTER(SCFOpts), C.c_int, C.POINTER(UHFResultC)]),
        "gbhf_scf_trace": (st, [_vp, _dp, C.c_int, _ip]),
        "gbhf_diis_error": (st, [_vp, C.c_int, _dp, _dp, _dp, _dp, _dp]),
        "gbhf_diis_extrapolate": (st, [_vp, C.c_int, C.c_int, _dp, _dp, _dp, _ip]),
        "gbhf_gauss_elem": (st, [_vp, C.c_int, _dp, _dp, _dp]),
        "gbhf_scf_opts_reference": (None, [C.POINTER(SCFOpts)]),
        "gbhf_scf_opts_baseline": (None, [C.POINTER(SCFOpts)]),
        "gbhf_scf": (st, [_vp, C.POINTER(SCFOpts), C.POINTER(SCFResultC)]),
        "gbhf_gradient": (st, [_vp, C.c_int, C.c_double, _dp, _dp, _dp]),
        "gbhf_gradient_uhf": (st, [_vp, C.c_int, C.c_double, _dp, _dp, _dp, _dp]),
        "gbhf_scf_batch": (st, [_vp, C.c_int, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _dp, _dp, C.POINTER(SCFOpts),
                                _dp, _ip, _ip, _dp]),
        "gbhf_profile_reset": (st, [_vp, C.c_int]),
        "gbhf_profile_read": (st, [_vp, _dp, C.c_int]),
        "gbhf_profile_classes": (st, [_vp, _dp]),
        "gbhf_event_record": (st, [_vp, C.c_int]),
        "gbhf_event_elapsed": (st, [_vp, C.c_int, C.c_int, _dp]),
        "gbhf_flush_l2": (st, [_vp]),
        "gbhf_peak_flops": (st, [_vp, C.c_int, _dp]),
        "gbhf_get_task_budgets": (st, [_vp, C.c_int, _ip, C.c_int]),
        "gbhf_set_task_budgets": (st, [_vp, C.c_int, _ip, C.c_int]),
        "gbhf_autotune": (st, [_vp, C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_int, _dp]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def declared_symbols():
    """Function names declared in include/gbhf.h."""
    import re
    text = re.sub(r"/\*.*?\*/", " ", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(gbhf_[a-z0-9_]+)\s*\(", text)))


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def reference_opts(**kw):
    o = SCFOpts()
    load().gbhf_scf_opts_reference(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def baseline_opts(**kw):
    o = SCFOpts()
    load().gbhf_scf_opts_baseline(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Context:
    """One libgbhf context (device memory + stream) on ``device``."""

    def __init__(self, device=0):
        self.L = load()
        h = _vp()
        s = self.L.gbhf_create(C.byref(h), int(device))
        if s != 0:
            raise GBHFError(s, "gbhf_create failed (no usable GPU?)")
        self.h = h
        self.n = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.gbhf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, s):
        if s != 0:
            msg = self.L.gbhf_last_error(self.h).decode(errors="replace")
            if s == 2:
                raise NotConverged(s, msg)
            raise GBHFError(s, msg)

    # -- basis ------------------------------------------------------------
    def set_basis(self, fb):
        self._keep = [_f64(fb.xyz.ravel()), _f64(fb.charge), np.ascontiguousarray(fb.cgf_atom, np.int32),
                      np.ascontiguousarray(fb.cgf_lxyz.ravel(), np.int32),
                      np.ascontiguousarray(fb.cgf_nprim, np.int32), _f64(fb.prim_coef), _f64(fb.prim_exp)]
        k = self._keep
        self._check(self.L.gbhf_set_basis(self.h, int(fb.n_atoms), _d(k[0]), _d(k[1]), int(fb.n_cgf), _i(k[2]),
                                          _i(k[3]), _i(k[4]), _d(k[5]), _d(k[6])))
        self.n = int(fb.n_cgf)
        return self

    @property
    def ntri(self):
        return self.n * (self.n + 1) // 2

    def set_boys_grid(self, grid):
        g = _f64(grid).ravel()
        assert g.size == 15 * 1001
        self._check(self.L.gbhf_set_boys_grid(self.h, _d(g)))

    def generate_boys_grid(self):
        g = np.zeros(15 * 1001)
        self._check(self.L.gbhf_generate_boys_grid(self.h, _d(g)))
        return g.reshape(15, 1001)

    def boys(self, mode, m_max, x):
        x = _f64(x).ravel()
        out = np.zeros((x.size, m_max + 1))
        self._check(self.L.gbhf_boys(self.h, mode, m_max, x.size, _d(x), _d(out)))
        return out

    # -- integrals --------------------------------------------------------
    def overlap(self, mode=MODE_REFERENCE):
        out = np.zeros(self.ntri)
        self._check(self.L.gbhf_overlap(self.h, mode, _d(out)))
        return out

    def hcore(self, mode=MODE_REFERENCE):
        out = np.zeros(self.ntri)
        self._check(self.L.gbhf_hcore(self.h, mode, _d(out)))
        return out

    def eri_canonical(self, mode=MODE_REFERENCE):
        n = self.L.gbhf_eri_canonical_length(self.n)
        out = np.zeros(n)
        self._check(self.L.gbhf_eri_canonical(self.h, mode, _d(out), n))
        return out

    def fock(self, h_flat, d_flat, mode=MODE_EXACT, precision=PREC_FP64, schwarz=1e-12, mixed=1e-4):
        h, d = _f64(h_flat), _f64(d_flat)
        out = np.zeros(self.ntri)
        self._check(self.L.gbhf_fock(self.h, mode, precision, schwarz, mixed, _d(h), _d(d), _d(out)))
        return out

    # -- dense linear algebra --------------------------------------------
    def symm_ortho(self, s_square):
        s = _f64(s_square)
        n = s.shape[0]
        x = np.zeros((n, n))
        self._check(self.L.gbhf_symm_ortho(self.h, n, _d(s), _d(x)))
        return x

    def eigen_solve(self, a_square):
        a = _f64(a_square)
        n = a.shape[0]
        w, v = np.zeros(n), np.zeros((n, n))
        self._check(self.L.gbhf_eigen_solve(self.h, n, _d(a), _d(w), _d(v)))
        return w, v

    def diagonal_hf(self, f_flat, x_square, n_occupied):
        f, x = _f64(f_flat), _f64(x_square)
        n = x.shape[0]
        c, d, e = np.zeros((n, n)), np.zeros(n * (n + 1) // 2), np.zeros(n)
        self._check(self.L.gbhf_diagonal_hf(self.h, n, _d(f), _d(x), int(n_occupied), _d(c), _d(d), _d(e)))
        return c, d, e

    def sad_density(self):
        """Superposition-of-atomic-densities starting density (flat upper triangle)."""
        d = np.zeros(self.n * (self.n + 1) // 2)
        self._check(self.L.gbhf_sad_density(self.h, _d(d)))
        return d

    def scf_uhf(self, multiplicity, opts=None, want_matrices=True):
        """Unrestricted SCF of the current basis for ``multiplicity`` (2S+1)."""
        opts = opts or baseline_opts()
        res = UHFResultC()
        keep = []
        if want_matrices:
            da, db = np.zeros(self.ntri), np.zeros(self.ntri)
            ea, eb = np.zeros(self.n), np.zeros(self.n)
            res.density_alpha_flat, res.density_beta_flat = _d(da), _d(db)
            res.orb_energies_alpha, res.orb_energies_beta = _d(ea), _d(eb)
            keep = [da, db, ea, eb]
        self._check(self.L.gbhf_scf_uhf(self.h, C.byref(opts), int(multiplicity), C.byref(res)))
        out = dict(energy=res.energy, iterations=res.iterations, converged=bool(res.converged),
                   n_alpha=res.n_alpha, n_beta=res.n_beta, s2=res.s2)
        if want_matrices:
            out.update(density_alpha=keep[0], density_beta=keep[1], orb_energies_alpha=keep[2],
                       orb_energies_beta=keep[3])
        return out

    def set_guess_density(self, d_flat):
        """Starting density (flat upper triangle) for an SCF with GUESS_DENSITY (restart)."""
        d = _f64(d_flat)
        if d.size != self.n * (self.n + 1) // 2:
            raise ValueError("density size does not match the basis")
        self._check(self.L.gbhf_set_guess_density(self.h, _d(d)))

    TRACE_KEYS = ("step", "energy", "delta_e", "rms_delta_d", "max_diis_error", "diis_vectors", "phase", "ms")

    def scf_trace(self):
        """Per-step records of the last SCF: list of dicts (TRACE_KEYS; phase 0 FP64,
        1 mixed, 2 FP64 after a mixed phase)."""
        nrec = C.c_int(0)
        self._check(self.L.gbhf_scf_trace(self.h, None, 0, C.byref(nrec)))
        out = np.zeros(max(nrec.value, 1) * len(self.TRACE_KEYS))
        self._check(self.L.gbhf_scf_trace(self.h, _d(out), nrec.value, C.byref(nrec)))
        recs = out[:nrec.value * len(self.TRACE_KEYS)].reshape(-1, len(self.TRACE_KEYS))
        return [dict(zip(self.TRACE_KEYS, r.tolist())) for r in recs]

    def diis_error(self, f_flat, s_flat, d_flat, x_square):
        x = _f64(x_square)
        n = x.shape[0]
        e = np.zeros((n, n))
        self._check(self.L.gbhf_diis_error(self.h, n, _d(_f64(f_flat)), _d(_f64(s_flat)), _d(_f64(d_flat)),
                                           _d(x), _d(e)))
        return e

    def diis_extrapolate(self, errors, focks):
        es = _f64(np.stack(errors))
        fs = _f64(np.stack(focks))
        n = es.shape[1]
        out = np.zeros(fs.shape[1])
        used = C.c_int(0)
        self._check(self.L.gbhf_diis_extrapolate(self.h, n, len(errors) - 1, _d(es), _d(fs), _d(out),
                                                 C.byref(used)))
        return out, used.value

    def gauss_elem(self, a, b):
        a, b = _f64(a), _f64(b)
        x = np.zeros(b.size)
        self._check(self.L.gbhf_gauss_elem(self.h, b.size, _d(a), _d(b), _d(x)))
        return x

    # -- SCF --------------------------------------------------------------
    def scf(self, opts=None, want_matrices=True):
        opts = opts or reference_opts()
        n = self.n
        bufs = {}
        r = SCFResultC()
        if want_matrices:
            bufs = dict(fock=np.zeros(self.ntri), coeff=np.zeros((n, n)), density=np.zeros(self.ntri),
                        orb_energies=np.zeros(n))
            r.fock_flat, r.coeff = _d(bufs["fock"]), _d(bufs["coeff"])
            r.density_flat, r.orb_energies = _d(bufs["density"]), _d(bufs["orb_energies"])
        s = self.L.gbhf_scf(self.h, C.byref(opts), C.byref(r))
        out = dict(energy=r.energy, iterations=r.iterations, converged=bool(r.converged),
                   n_occupied=r.n_occupied, nuclear_repulsion=r.nuclear_repulsion,
                   eri_quartets=r.eri_quartets, eri_fn_quartets=r.eri_fn_quartets,
                   eri_prim_quartets=r.eri_prim_quartets, eri_fp32_fraction=r.eri_fp32_fraction,
                   fock_builds=r.fock_builds, status=s)
        out.update(bufs)
        self._check(s)
        return out

    def scf_batch(self, flats, opts=None, gradients=False):
        """SCF of many molecules (list of FlatBasis) in one call; returns
        (energies, iterations, converged, gradients or None)."""
        opts = opts or baseline_opts()
        ao, co = [0], [0]
        xyz, z, catom, lx, npr, pc, pe = [], [], [], [], [], [], []
        for fb in flats:
            catom.append(np.asarray(fb.cgf_atom, np.int32) + ao[-1])
            ao.append(ao[-1] + int(fb.n_atoms))
            co.append(co[-1] + int(fb.n_cgf))
            xyz.append(fb.xyz.ravel()); z.append(fb.charge); lx.append(fb.cgf_lxyz.ravel())
            npr.append(fb.cgf_nprim); pc.append(fb.prim_coef); pe.append(fb.prim_exp)
        arrs = [np.asarray(ao, np.int32), np.asarray(co, np.int32), _f64(np.concatenate(xyz)),
                _f64(np.concatenate(z)), np.ascontiguousarray(np.concatenate(catom), np.int32),
                np.ascontiguousarray(np.concatenate(lx), np.int32),
                np.ascontiguousarray(np.concatenate(npr), np.int32), _f64(np.concatenate(pc)),
                _f64(np.concatenate(pe))]
        nm = len(flats)
        e = np.zeros(nm)
        it = np.zeros(nm, np.int32)
        cv = np.zeros(nm, np.int32)
        g = np.zeros(3 * ao[-1]) if gradients else None
        s = self.L.gbhf_scf_batch(self.h, nm, _i(arrs[0]), _i(arrs[1]), _d(arrs[2]), _d(arrs[3]), _i(arrs[4]),
                                  _i(arrs[5]), _i(arrs[6]), _d(arrs[7]), _d(arrs[8]), C.byref(opts), _d(e), _i(it),
                                  _i(cv), _d(g) if gradients else None)
        self.n = 0          # the context now holds the batch's basis
        self._keep = None
        self._check(s)
        grads = [g[3 * ao[k]:3 * ao[k + 1]].reshape(-1, 3) for k in range(nm)] if gradients else None
        return e, it, cv.astype(bool), grads

    def gradient(self, d_flat=None, w_flat=None, schwarz=1e-12, precision=PREC_FP64, n_atoms=None):
        """dE/dR (n_atoms, 3) in hartree/bohr.  Without D and W: the last SCF's."""
        na = n_atoms if n_atoms is not None else self._keep[1].size
        g = np.zeros(3 * na)
        if d_flat is None:
            s = self.L.gbhf_gradient(self.h, precision, schwarz, None, None, _d(g))
        else:
            d, w = _f64(d_flat), _f64(w_flat)
            s = self.L.gbhf_gradient(self.h, precision, schwarz, _d(d), _d(w), _d(g))
        self._check(s)
        return g.reshape(na, 3)

    def gradient_uhf(self, da_flat=None, db_flat=None, w_flat=None, schwarz=1e-12, precision=PREC_FP64):
        """Open-shell dE/dR (n_atoms, 3) in hartree/bohr.  Without densities:
        the last converged UHF SCF of this basis."""
        na = self._keep[1].size
        g = np.zeros(3 * na)
        if da_flat is None:
            s = self.L.gbhf_gradient_uhf(self.h, precision, schwarz, None, None, None, _d(g))
        else:
            da, db, w = _f64(da_flat), _f64(db_flat), _f64(w_flat)
            s = self.L.gbhf_gradient_uhf(self.h, precision, schwarz, _d(da), _d(db), _d(w), _d(g))
        self._check(s)
        return g.reshape(na, 3)

    # -- measurement ------------------------------------------------------
    def profile_reset(self, events=True):
        self._check(self.L.gbhf_profile_reset(self.h, 1 if events else 0))

    def profile_read(self):
        v = np.zeros(20)
        self._check(self.L.gbhf_profile_read(self.h, _d(v), 20))
        keys = ("jk_ms_fp64", "jk_ms_fp32", "prim_quartets_fp64", "prim_quartets_fp32", "shell_quartets",
                "fn_quartets", "launches", "dense_ms", "ms_setup", "ms_fock", "ms_diis", "ms_diag", "ms_other",
                "jacobi_sweeps", "jacobi_calls", "ms_grad", "batch_steps", "purify_steps", "purify_calls", "ms_pairs")
        return dict(zip(keys, v.tolist()))

    CLASSES = ("ssss", "psss", "psps", "ppss", "ppps", "pppp", "dsss", "dsps", "dspp", "dsds", "dpss", "dpps",
               "dppp", "dpds", "dpdp", "ddss", "ddps", "ddpp", "ddds", "dddp", "dddd")

    def profile_classes(self):
        """{(class, 'fp64'|'fp32'): dict(shell_quartets, fn_quartets, prim_quartets, ms)}"""
        v = np.zeros(8 * len(self.CLASSES))
        self._check(self.L.gbhf_profile_classes(self.h, _d(v)))
        out = {}
        for k, name in enumerate(self.CLASSES):
            for p, prec in enumerate(("fp64", "fp32")):
                q = v[(k * 2 + p) * 4:(k * 2 + p) * 4 + 4]
                out[(name, prec)] = dict(shell_quartets=q[0], fn_quartets=q[1], prim_quartets=q[2], ms=q[3])
        return out

    def event_record(self, slot):
        self._check(self.L.gbhf_event_record(self.h, slot))

    def event_elapsed(self, a, b):
        ms = C.c_double(0)
        self._check(self.L.gbhf_event_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value

    def flush_l2(self):
        self._check(self.L.gbhf_flush_l2(self.h))

    # -- task budgets and the autotuner --------------------------------------
    GRAD_PAIRS = ("ss", "ps", "pp", "ds", "dp", "dd")

    def budget_classes(self, which):
        """Class names of the budget table: J/K quartet classes (which 0) or
        gradient (bra pair class, ket pair class) combinations (which 1)."""
        if which == 0:
            return self.CLASSES
        return tuple(f"{a}|{b}" for a in self.GRAD_PAIRS for b in self.GRAD_PAIRS)

    def task_budgets(self, which=0):
        """int array (classes, 2): primitive quartets per lane, kets per task."""
        n = len(self.budget_classes(which))
        v = np.zeros(2 * n, dtype=np.int32)
        self._check(self.L.gbhf_get_task_budgets(self.h, which, _i(v), 2 * n))
        return v.reshape(n, 2)

    def set_task_budgets(self, which, budgets=None):
        """Set the budget table (classes, 2), or restore the defaults (None)."""
        n = len(self.budget_classes(which))
        if budgets is None:
            self._check(self.L.gbhf_set_task_budgets(self.h, which, None, 2 * n))
            return
        v = np.ascontiguousarray(budgets, dtype=np.int32).reshape(-1)
        self._check(self.L.gbhf_set_task_budgets(self.h, which, _i(v), v.size))

    def autotune(self, which=0, precision=PREC_MIXED, schwarz=1e-12, mixed=1e-4, d_flat=None, repeats=2):
        """Tune the budgets on the current basis; returns (ms before, ms after) per class."""
        n = len(self.budget_classes(which))
        ms = np.zeros(2 * n)
        dd = None if d_flat is None else _f64(d_flat)
        d = None if dd is None else _d(dd)
        self._check(self.L.gbhf_autotune(self.h, which, precision, schwarz, mixed, d, repeats, _d(ms)))
        ms = ms.reshape(n, 2)
        return ms[:, 0].copy(), ms[:, 1].copy()

    def peak_flops(self, precision):
        t = C.c_double(0)
        self._check(self.L.gbhf_peak_flops(self.h, precision, C.byref(t)))
        return t.value
