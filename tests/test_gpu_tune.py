"""Task budgets and the autotuner: any budget table gives the same Fock
matrices and gradients (the budgets only split the work into tasks), the
autotuner keeps valid tables and never slows a class down by its own
measure, and the batched driver's autotune option leaves its results as they
were."""
import numpy as np
import pytest

import oracle as O
from gbhf import _lib, basis as B, molecules as M

pytestmark = pytest.mark.gpu


@pytest.fixture
def tctx(ctx):
    """The session context, with default budgets restored afterwards."""
    yield ctx
    ctx.set_task_budgets(0, None)
    ctx.set_task_budgets(1, None)


def _rand_density(n, seed, scale=0.05):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((n, n)) * scale
    return O.square_to_tri(d + d.T)


def test_default_tables(tctx):
    jk = tctx.task_budgets(0)
    gr = tctx.task_budgets(1)
    assert jk.shape == (21, 2) and gr.shape == (36, 2)
    assert (jk[:, 0] >= 1).all() and (gr[:, 0] >= 1).all()
    assert set(jk[:, 1]) <= {1, 32} and set(gr[:, 1]) <= {1, 32}
    assert (jk[:6, 1] == 32).all()   # the s/p classes: a lane per ket


def test_bad_budgets_rejected(tctx):
    b = tctx.task_budgets(0)
    for (row, col, value) in ((0, 0, 0), (3, 1, 0), (5, 1, 33), (2, 0, 70000)):
        t = b.copy()
        t[row, col] = value
        with pytest.raises(_lib.GBHFError) as ei:
            tctx.set_task_budgets(0, t)
        assert ei.value.name == "GBHF_ERR_BAD_INPUT"
    with pytest.raises(_lib.GBHFError):
        tctx.set_task_budgets(2, b)
    np.testing.assert_array_equal(tctx.task_budgets(0), b)


@pytest.mark.parametrize("basis", ["6-31g", "6-31g*"])
def test_fock_independent_of_budgets(tctx, basis):
    """(H2O)4: FP64 and mixed Fock matrices with extreme budget tables (one
    primitive quartet per lane; 64x the default; one ket per task everywhere;
    8 kets per task for the warp-per-quartet classes) equal the default ones."""
    fb = B.flatten(M.cluster_atoms("batch256", basis, index=20))
    tctx.set_basis(fb)
    h = O.OracleBasis(fb).hcore(False)
    d = _rand_density(fb.n_cgf, 5)
    ref64 = tctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_FP64, 1e-12, 0.0)
    refmx = tctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_MIXED, 1e-12, 1e-4)
    base = tctx.task_budgets(0)
    tables = []
    t = base.copy(); t[:, 0] = 1; tables.append(t)
    t = base.copy(); t[:, 0] = np.minimum(base[:, 0] * 64, 65535); tables.append(t)
    t = base.copy(); t[:, 1] = 1; tables.append(t)
    t = base.copy(); t[base[:, 1] < 32, 1] = 8; tables.append(t)
    for t in tables:
        tctx.set_task_budgets(0, t)
        np.testing.assert_array_equal(tctx.task_budgets(0), t)
        f64 = tctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_FP64, 1e-12, 0.0)
        np.testing.assert_allclose(f64, ref64, rtol=0, atol=1e-12)
        # FP32 partial sums per task depend on the split: a fraction of the
        # 1e-6 mixed-vs-FP64 bound
        fmx = tctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_MIXED, 1e-12, 1e-4)
        np.testing.assert_allclose(fmx, refmx, rtol=0, atol=1e-7)


def test_gradient_independent_of_budgets(tctx):
    """(H2O)2/6-31G*: the analytic gradient with one primitive quartet per lane
    and one ket per task equals the default-table gradient."""
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g*", index=7))
    tctx.set_basis(fb)
    tctx.scf(_lib.baseline_opts(conv_energy=1e-12, conv_density=1e-10), want_matrices=False)
    g0 = tctx.gradient()
    t = tctx.task_budgets(1)
    t[:, 0] = 1
    t[:, 1] = 1
    tctx.set_task_budgets(1, t)
    g1 = tctx.gradient()
    np.testing.assert_allclose(g1, g0, rtol=0, atol=1e-11)


@pytest.mark.parametrize("which", [0, 1])
def test_autotune_keeps_results(tctx, which):
    """(H2O)4/6-31G*: the tuned table is valid, no class got slower by the
    tuner's own measure, and the Fock matrix / gradient is unchanged."""
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g*", index=20))
    tctx.set_basis(fb)
    h = O.OracleBasis(fb).hcore(False)
    if which == 0:
        d = _rand_density(fb.n_cgf, 9)
        before = tctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_MIXED, 1e-12, 1e-4)
    else:
        tctx.scf(_lib.baseline_opts(conv_energy=1e-12, conv_density=1e-10), want_matrices=False)
        before = tctx.gradient(precision=_lib.PREC_MIXED)
    ms0, ms1 = tctx.autotune(which, _lib.PREC_MIXED, 1e-12, 1e-4, None, 2)
    assert (ms1 <= ms0 + 1e-9).all()
    assert ms0.sum() > 0
    t = tctx.task_budgets(which)
    assert (t[:, 0] >= 1).all() and (t[:, 1] >= 1).all() and (t[:, 1] <= 32).all()
    if which == 0:
        after = tctx.fock(h, d, _lib.MODE_EXACT, _lib.PREC_MIXED, 1e-12, 1e-4)
        np.testing.assert_allclose(after, before, rtol=0, atol=1e-7)
    else:
        after = tctx.gradient(precision=_lib.PREC_MIXED)
        np.testing.assert_allclose(after, before, rtol=0, atol=1e-7)


def test_batch_autotune_option(tctx):
    """gbhf_scf_batch with autotune = 1: the same energies and gradients as
    without, and tuned tables left in the context."""
    picks = [(1, "6-31g"), (2, "sto-3g"), (3, "6-31g*"), (8, "6-31g")]
    flats = [B.flatten(M.cluster_atoms("batch256", b, index=i)) for i, b in picks]
    opts = _lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1)
    e0, _, cv0, g0 = tctx.scf_batch(flats, opts, gradients=True)
    d0 = (tctx.task_budgets(0).copy(), tctx.task_budgets(1).copy())
    opts.autotune = 1
    e1, _, cv1, g1 = tctx.scf_batch(flats, opts, gradients=True)
    assert cv0.all() and cv1.all()
    np.testing.assert_allclose(e1, e0, rtol=0, atol=1e-8)
    for a, b in zip(g1, g0):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-7)
    t = (tctx.task_budgets(0), tctx.task_budgets(1))
    for x in t:
        assert (x[:, 0] >= 1).all() and (x[:, 1] >= 1).all() and (x[:, 1] <= 32).all()
    assert t[0].shape == d0[0].shape and t[1].shape == d0[1].shape
