"""The three multi-molecule workloads, each checked against the FP64 oracle or
against central finite differences, at the tolerances the workloads state.

* (H2O)8 RHF/6-31G analytic gradient (104 functions): FP64 gradient against
  central differences (h = 1e-4 bohr) of the GPU SCF energy on all 72
  Cartesian coordinates (1e-6 Eh/bohr) and against central differences of the
  oracle's energies on three coordinates; mixed-precision gradient within
  1e-5 Eh/bohr of FP64.  The reference's own gradient (Derivatives.hs:40-48)
  is dead code, so the specification is the derivative of the SCF energy of
  scfHF (HartreeFock.hs:70-123).
* Batched SCF of uneven conformers (STO-3G even index, 6-31G odd): mixed
  batched energies within 1e-6 Eh of the oracle's FP64 energies, batched mixed
  gradients within 1e-5 Eh/bohr of the FP64 gradient and of central
  differences of oracle energies, at the Schwarz-bound cutoffs the
  batch benchmark uses and at 1e-4.
* (H2O)64 RHF/6-31G (832 functions), the large direct SCF that replaces
  stored integrals (HartreeFock.hs:166-181 stores all N^4/8): mixed within
  1e-6 Eh of the FP64 GPU SCF, mixed gradient within 1e-5 Eh/bohr.
"""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu

H = 1e-4
TIGHT = dict(conv_energy=1e-12, conv_density=1e-10, max_iter=200)


def _flat(labels, xyz, basis):
    return B.flatten(B.make_atoms(labels, xyz, basis, "text"))


def _gpu_energy(ctx, labels, xyz, basis):
    ctx.set_basis(_flat(labels, xyz, basis))
    return ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)["energy"]


def _oracle_fd(labels, xyz, basis, coords):
    """Central differences of the oracle's FP64 SCF energy; every displaced SCF
    starts from the oracle's converged density at ``xyz``."""
    o0 = O.scf(_flat(labels, xyz, basis), O.SCFOptions.baseline(guess="sad", **TIGHT))
    out = {}
    for (a, x) in coords:
        e = []
        for s in (1, -1):
            p = xyz.copy()
            p[a, x] += s * H
            e.append(O.scf(_flat(labels, p, basis),
                           O.SCFOptions.baseline(guess="density", guess_density=o0.density, **TIGHT)).energy)
        out[(a, x)] = (e[0] - e[1]) / (2 * H)
    return o0, out


def test_w8_gradient_all_72_coordinates(ctx):
    xyz = M.cluster_coords("w8")
    labels = M.water_labels(len(xyz) // 3)
    assert len(xyz) * 3 == 72
    ctx.set_basis(_flat(labels, xyz, "6-31g"))
    r64 = ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)
    g64 = ctx.gradient()
    assert np.max(np.abs(g64.sum(axis=0))) < 1e-8
    ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, **TIGHT), want_matrices=False)
    gmx = ctx.gradient(precision=_lib.PREC_MIXED)
    assert np.max(np.abs(gmx - g64)) <= 1e-5
    worst = 0.0
    for idx in range(72):
        a, x = divmod(idx, 3)
        e = []
        for s in (1, -1):
            p = xyz.copy()
            p[a, x] += s * H
            e.append(_gpu_energy(ctx, labels, p, "6-31g"))
        fd = (e[0] - e[1]) / (2 * H)
        worst = max(worst, abs(fd - g64[a, x]))
        assert abs(fd - g64[a, x]) < 1e-6, ((a, x), g64[a, x], fd)
    # the oracle: its energy at the centre, and its own finite differences
    coords = [(0, 0), (1, 2), (16, 1)]
    o0, fd_o = _oracle_fd(labels, xyz, "6-31g", coords)
    assert abs(o0.energy - r64["energy"]) < 1e-8
    for k, v in fd_o.items():
        assert abs(g64[k] - v) < 1e-6, (k, g64[k], v)


BATCH = list(range(12)) + [15, 38]          # 1..12 waters; 15 and 38 are single waters
ORACLE_MEMBERS = (2, 3, 6, 7, 15, 38)       # 2, 4, 6, 2, 1, 1 waters (STO-3G even, 6-31G odd)


@pytest.fixture(scope="module")
def batch_inputs():
    flats = []
    for i in BATCH:
        basis = "sto-3g" if i % 2 == 0 else "6-31g"
        flats.append(B.flatten(M.cluster_atoms("batch256", basis, index=i)))
    oracle_e = {i: O.scf(flats[BATCH.index(i)], O.SCFOptions.baseline(guess="sad", **TIGHT)).energy
                for i in ORACLE_MEMBERS}
    return flats, oracle_e


# (FP32 cutoff for ERIs, for derivative ERIs): the batch benchmark's settings and 1e-4
@pytest.mark.parametrize("cut,gcut", [(1e-2, 1.0), (1e-4, 1e-4)], ids=["bench-cutoffs", "1e-4"])
def test_batch_mixed_against_oracle(ctx, batch_inputs, cut, gcut):
    flats, oracle_e = batch_inputs
    opts = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, final_fp64=0, full_rebuild_every=0,
                              mixed_cutoff=cut, grad_mixed_cutoff=gcut)
    e, it, cv, grads = ctx.scf_batch(flats, opts, gradients=True)
    assert cv.all()
    for i, eo in oracle_e.items():
        k = BATCH.index(i)
        assert abs(e[k] - eo) <= 1e-6, (i, e[k], eo)
    # mixed batched gradients against the FP64 one-molecule gradient
    for i in ORACLE_MEMBERS:
        k = BATCH.index(i)
        ctx.set_basis(flats[k])
        ctx.scf(_lib.baseline_opts(**TIGHT), want_matrices=False)
        g64 = ctx.gradient()
        assert np.max(np.abs(grads[k] - g64)) <= 1e-5, i
        # translational invariance, to the FP32 rounding of the derivative integrals
        assert np.max(np.abs(grads[k].sum(axis=0))) < 1e-6


def test_batch_gradient_against_oracle_fd(ctx, batch_inputs):
    """Single-water members of the batch (6-31G and STO-3G): the batched mixed
    gradient against central differences of the oracle's energies on all nine
    coordinates."""
    flats, _ = batch_inputs
    opts = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, final_fp64=0, full_rebuild_every=0,
                              mixed_cutoff=1e-2, grad_mixed_cutoff=1.0)
    e, it, cv, grads = ctx.scf_batch(flats, opts, gradients=True)
    for i in (15, 38):
        k = BATCH.index(i)
        basis = "sto-3g" if i % 2 == 0 else "6-31g"
        xyz = M.cluster_coords("batch256", i)
        _, fd = _oracle_fd(["O", "H", "H"], xyz, basis, [(a, x) for a in range(3) for x in range(3)])
        for key, v in fd.items():
            assert abs(grads[k][key] - v) <= 1e-5, (i, key, grads[k][key], v)


def test_w64_mixed_against_fp64():
    """(H2O)64/6-31G on its own context (the largest basis of the suite)."""
    fb = B.flatten(M.cluster_atoms("w64", "6-31g"))
    assert fb.n_cgf == 832
    with _lib.Context(0) as c:
        c.set_basis(fb)
        r64 = c.scf(_lib.baseline_opts(), want_matrices=False)
        g64 = c.gradient()
        c.set_basis(fb)
        rmx = c.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1), want_matrices=False)
        gmx = c.gradient(precision=_lib.PREC_MIXED)
    assert r64["converged"] and rmx["converged"]
    assert abs(rmx["energy"] - r64["energy"]) <= 1e-6
    assert rmx["eri_fp32_fraction"] > 0.5
    assert np.max(np.abs(gmx - g64)) <= 1e-5
    assert np.max(np.abs(g64.sum(axis=0))) < 1e-7
    assert np.max(np.abs(gmx.sum(axis=0))) < 1e-6
