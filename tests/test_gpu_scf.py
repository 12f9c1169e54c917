"""Full SCF on the device versus the oracle driver."""
import numpy as np
import pytest

import oracle as O
from conftest import golden
from gbhf import _lib, basis as B, hartree_fock as HF, molecules as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", ["shipped", "text"])
def test_water_sto3g_reference_mode_energy(ctx, variant):
    """H2O/STO-3G with the reference's numerics and driver: within 1e-8 Eh of the
    oracle (and of the committed golden energy)."""
    fb = B.flatten(M.water_atoms("sto-3g", variant))
    ctx.set_basis(fb)
    ctx.generate_boys_grid()
    r = ctx.scf(_lib.reference_opts())
    o = O.scf(fb, O.SCFOptions.reference())
    assert abs(r["energy"] - o.energy) < 1e-8
    assert abs(r["energy"] - golden("water_sto3g.json")[variant]["energy_reference_driver"]) < 1e-8
    assert r["iterations"] == o.iterations
    np.testing.assert_allclose(r["density"], o.density, rtol=0, atol=1e-7)
    np.testing.assert_allclose(r["orb_energies"], o.orb_energies, rtol=0, atol=1e-7)


def test_water_sto3g_config_options(ctx):
    """The single-water workload's stated options (reference numerics, Harris
    guess, DIIS with 6 vectors, dE < 1e-10, RMS dD < 1e-8) agree with the
    oracle run the same way to 1e-10 Eh.  The reference's own stop rule
    (max|e| < 1e-7, energy from F_DIIS and the new density) lands 3.5e-8 Eh
    away from that converged energy, which bounds how closely the two rules
    can agree."""
    fb = B.flatten(M.water_atoms("sto-3g", "shipped"))
    ctx.set_basis(fb)
    ctx.generate_boys_grid()
    r_ref = ctx.scf(_lib.reference_opts())
    opts = _lib.reference_opts(diis_size=6, ref_stop_rule=0, conv_energy=1e-10, conv_density=1e-8)
    r = ctx.scf(opts)
    o = O.scf(fb, O.SCFOptions(ref_compat=True, guess="harris", diis_size=6, stop_rule="energy"))
    assert abs(r["energy"] - o.energy) < 1e-10
    assert abs(r["energy"] - r_ref["energy"]) < 1e-7


def test_mirror_scf_hf(ctx):
    atoms = M.water_atoms("sto-3g", "shipped")
    hf = HF.scf_hf(atoms, 0.0)
    assert abs(hf.energy - golden("water_sto3g.json")["shipped"]["energy_reference_driver"]) < 1e-8
    assert hf.coeff.shape == (7, 7) and hf.density.shape == (28,)


SYSTEMS = [
    ("water 6-31g", lambda: M.water_atoms("6-31g", "text")),
    ("(H2O)2 6-31g", lambda: M.cluster_atoms("batch256", "6-31g", index=7)),
    ("(H2O)4 sto-3g", lambda: M.cluster_atoms("batch256", "sto-3g", index=20)),
]


@pytest.mark.parametrize("name,make", SYSTEMS, ids=[s[0] for s in SYSTEMS])
def test_exact_mode_fp64_energy(ctx, name, make):
    fb = B.flatten(make())
    ctx.set_basis(fb)
    r = ctx.scf(_lib.baseline_opts())
    o = O.scf(fb, O.SCFOptions.baseline())
    assert abs(r["energy"] - o.energy) < 1e-8
    np.testing.assert_allclose(r["density"], o.density, rtol=0, atol=1e-6)


def test_cluster_fixture_energies(ctx):
    for name, rec in golden("clusters.json").items():
        if "batch_index" in rec:
            atoms = M.cluster_atoms("batch256", rec["basis"], index=rec["batch_index"])
        else:
            atoms = M.cluster_atoms(rec["cluster"], rec["basis"])
        ctx.set_basis(B.flatten(atoms))
        r = ctx.scf(_lib.baseline_opts(), want_matrices=False)
        assert abs(r["energy"] - rec["energy"]) < 1e-8, name
        # mixed precision (FP32 below Schwarz bound 1e-4, incremental builds) within 1e-6
        rm = ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1), want_matrices=False)
        assert abs(rm["energy"] - rec["energy"]) < 1e-6, name


def test_mixed_precision_energy_w8(ctx):
    ctx.set_basis(B.flatten(M.cluster_atoms("w8", "6-31g")))
    r64 = ctx.scf(_lib.baseline_opts(), want_matrices=False)
    for inc in (0, 1):
        rmx = ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=inc), want_matrices=False)
        assert abs(rmx["energy"] - r64["energy"]) < 1e-6
        assert rmx["eri_fp32_fraction"] > 0.5


def test_harris_guess_out_of_bounds_like_reference(ctx):
    """The reference's Harris guess indexes outside the ERI array for 6-31G
    water (HartreeFock.hs:143-146); the library reports GBHF_ERR_INDEX."""
    ctx.set_basis(B.flatten(M.water_atoms("6-31g", "text")))
    ctx.generate_boys_grid()
    with pytest.raises(_lib.GBHFError) as e:
        ctx.scf(_lib.reference_opts())
    assert e.value.name == "GBHF_ERR_INDEX"


def test_not_converged_raises(ctx):
    ctx.set_basis(B.flatten(M.water_atoms("sto-3g", "text")))
    ctx.generate_boys_grid()
    with pytest.raises(_lib.NotConverged):
        ctx.scf(_lib.reference_opts(max_iter=2))


@pytest.mark.parametrize("basis,index", [("6-31g", 7), ("sto-3g", 20), ("sto-3g", 154)])
def test_sad_density_matches_oracle(ctx, basis, index):
    fb = B.flatten(M.cluster_atoms("batch256", basis, index=index))
    ctx.set_basis(fb)
    np.testing.assert_allclose(ctx.sad_density(), O.sad_density(fb), rtol=0, atol=1e-9)


def test_sad_guess_converges_where_core_guess_does_not(ctx):
    """Conformer 154 of the 256-molecule set, (H2O)7/STO-3G: the core guess with
    DIIS from the first step oscillates past 100 steps (oracle and library
    alike); the SAD guess converges to the oracle's energy."""
    fb = B.flatten(M.cluster_atoms("batch256", "sto-3g", index=154))
    ctx.set_basis(fb)
    with pytest.raises(_lib.NotConverged):
        ctx.scf(_lib.baseline_opts(guess=_lib.GUESS_CORE), want_matrices=False)
    r = ctx.scf(_lib.baseline_opts(), want_matrices=False)
    o = O.scf(fb, O.SCFOptions.baseline(guess="sad"))
    assert r["converged"] and abs(r["energy"] - o.energy) < 1e-8
    assert r["iterations"] <= 15


def test_restart_from_checkpoint_density_and_step_records(ctx):
    """GBHF_GUESS_DENSITY restarts from a stored density: from the converged
    density of an earlier run the SCF stops after two steps at the same energy.
    The per-step records describe each run (energies, phases)."""
    fb = B.flatten(M.cluster_atoms("batch256", "6-31g", index=7))
    ctx.set_basis(fb)
    r = ctx.scf(_lib.baseline_opts(guess=_lib.GUESS_SAD))
    tr = ctx.scf_trace()
    assert len(tr) == r["iterations"]
    assert [t["step"] for t in tr] == list(range(len(tr)))
    assert abs(tr[-1]["energy"] - r["energy"]) < 1e-12
    assert all(t["phase"] == 0 for t in tr) and all(t["ms"] > 0 for t in tr)
    assert tr[-1]["rms_delta_d"] < 1e-8 and abs(tr[-1]["delta_e"]) < 1e-10
    ctx.set_guess_density(r["density"])
    r2 = ctx.scf(_lib.baseline_opts(guess=_lib.GUESS_DENSITY))
    assert r2["iterations"] <= 2 and abs(r2["energy"] - r["energy"]) < 1e-9
    # mixed precision with the FP64 final phase: phases 1 then 2 in the records
    ctx.scf(_lib.baseline_opts(precision=_lib.PREC_MIXED, incremental=1, final_fp64=1), want_matrices=False)
    ph = [t["phase"] for t in ctx.scf_trace()]
    assert ph[0] == 1 and ph[-1] == 2 and sorted(ph) == ph
    # a new basis drops the stored density
    ctx.set_basis(B.flatten(M.water_atoms("sto-3g", "text")))
    with pytest.raises(_lib.GBHFError) as e:
        ctx.scf(_lib.baseline_opts(guess=_lib.GUESS_DENSITY))
    assert e.value.name == "GBHF_ERR_BAD_INPUT"
