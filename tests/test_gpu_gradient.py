"""Analytic RHF nuclear gradient (the backward call) against central finite
differences of the SCF energy (step 1e-4 bohr) on the device and in the
oracle, translational invariance, and the mixed-precision gradient error."""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu

H = 1e-4
TIGHT = dict(conv_energy=1e-12, conv_density=1e-10, max_iter=200)


def _atoms_at(labels, xyz, basis):
    return B.make_atoms(labels, xyz, basis, "text")


def _gpu_energy(ctx, labels, xyz, basis, **kw):
    ctx.set_basis(B.flatten(_atoms_at(labels, xyz, basis)))
    return ctx.scf(_lib.baseline_opts(**{**TIGHT, **kw}), want_matrices=False)["energy"]


def _fd(energy, xyz, coords):
    out = {}
    for (a, x) in coords:
        xp, xm = xyz.copy(), xyz.copy()
        xp[a, x] += H
        xm[a, x] -= H
        out[(a, x)] = (energy(xp) - energy(xm)) / (2 * H)
    return out


def _analytic(ctx, labels, xyz, basis, **kw):
    ctx.set_basis(B.flatten(_atoms_at(labels, xyz, basis)))
    ctx.scf(_lib.baseline_opts(**{**TIGHT, **kw}), want_matrices=False)
    return ctx.gradient()


def test_water_gradient_vs_finite_differences(ctx):
    labels, xyz = ["O", "H", "H"], M.WATER_BOHR.copy()
    xyz[1, 0] += 0.05   # break the symmetry a little
    g = _analytic(ctx, labels, xyz, "6-31g")
    assert np.max(np.abs(g.sum(axis=0))) < 1e-9   # translational invariance
    coords = [(a, x) for a in range(3) for x in range(3)]
    fd = _fd(lambda p: _gpu_energy(ctx, labels, p, "6-31g"), xyz, coords)
    for (a, x), v in fd.items():
        assert abs(g[a, x] - v) < 1e-6, ((a, x), g[a, x], v)
    # the FP64 oracle's energies give the same finite differences
    fd_o = _fd(lambda p: O.scf(B.flatten(_atoms_at(labels, p, "6-31g")),
                              O.SCFOptions.baseline(conv_energy=1e-12, conv_density=1e-10, max_iter=200)).energy,
               xyz, coords[:4])
    for k, v in fd_o.items():
        assert abs(g[k] - v) < 1e-6, (k, g[k], v)


def test_water_dimer_gradient_subset(ctx):
    xyz = M.cluster_coords("batch256", 7)
    labels = M.water_labels(len(xyz) // 3)
    g = _analytic(ctx, labels, xyz, "6-31g")
    assert np.max(np.abs(g.sum(axis=0))) < 1e-9
    coords = [(0, 0), (1, 2), (3, 1), (5, 0)]
    fd = _fd(lambda p: _gpu_energy(ctx, labels, p, "6-31g"), xyz, coords)
    for k, v in fd.items():
        assert abs(g[k] - v) < 1e-6, (k, g[k], v)


def test_gradient_with_explicit_density(ctx):
    """gbhf_gradient(D, W) with the caller's matrices equals the last-SCF path."""
    fb = B.flatten(M.water_atoms("sto-3g", "text"))
    ctx.set_basis(fb)
    r = ctx.scf(_lib.baseline_opts(**TIGHT))
    g_last = ctx.gradient()
    c, eps = r["coeff"], r["orb_energies"]
    nocc = r["n_occupied"]
    d = 2 * c[:, :nocc] @ c[:, :nocc].T
    w = 2 * (c[:, :nocc] * eps[:nocc]) @ c[:, :nocc].T
    g_dw = ctx.gradient(O.square_to_tri(d), O.square_to_tri(w))
    np.testing.assert_allclose(g_dw, g_last, rtol=0, atol=1e-8)


def test_mixed_precision_gradient_error(ctx):
    """(H2O)8 6-31G: gradient of the mixed-precision SCF within 1e-5 Eh/bohr of FP64."""
    fb = B.flatten(M.cluster_atoms("w8", "6-31g"))
    ctx.set_basis(fb)
    ctx.scf(_lib.baseline_opts(), want_matrices=False)
    g64 = ctx.gradient()
    ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1), want_matrices=False)
    gmx = ctx.gradient(precision=_lib.PREC_MIXED)
    assert np.max(np.abs(gmx - g64)) < 1e-5
    assert np.max(np.abs(g64.sum(axis=0))) < 1e-8
