"""gbhf_scf_batch: many molecules of uneven size in one call give the same
energies and gradients as one-at-a-time SCFs."""
import numpy as np
import pytest

from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu


def test_batch_matches_single_runs(ctx):
    confs = M._cluster_file()["batch256"]
    picks = list(range(12))            # STO-3G (even) and 6-31G (odd), 1..12 waters
    atoms = [M.cluster_atoms("batch256", "sto-3g" if i % 2 == 0 else "6-31g", index=i) for i in picks]
    flats = [B.flatten(a) for a in atoms]
    opts = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1)
    e, it, cv, grads = ctx.scf_batch(flats, opts, gradients=True)
    assert cv.all()
    for k in (0, 3, 7):
        ctx.set_basis(flats[k])
        r = ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1), want_matrices=False)
        assert abs(r["energy"] - e[k]) < 1e-8
        g = ctx.gradient()
        np.testing.assert_allclose(grads[k], g, rtol=0, atol=1e-7)
    for g in grads:
        assert np.max(np.abs(g.sum(axis=0))) < 1e-8
    assert len(confs) == 256


def test_batch_reports_failures(ctx):
    flats = [B.flatten(M.water_atoms("sto-3g", "text")), B.flatten(M.water_atoms("6-31g", "text"))]
    with pytest.raises(_lib.NotConverged):
        ctx.scf_batch(flats, _lib.baseline_opts(max_iter=2))
