"""The library on the reference's own sample inputs (HsFock/SampleProjects.hs:18-98:
HHe+, CO and water in STO-3G, water in 6-31G*), built from the literal
primitives and geometries in tests/golden/sample_projects.json, against the
oracle's energies on the same inputs."""
import sys

import pytest

import oracle as O
from conftest import GOLDEN, golden
from gbhf import _lib, basis as B

sys.path.insert(0, str(GOLDEN))
from make_golden import sample_atoms  # noqa: E402

pytestmark = pytest.mark.gpu

SAMPLES = golden("sample_projects.json")
D_ORDER = ("Dxx", "Dxy", "Dxz", "Dyy", "Dyz", "Dzz")   # createCGF (FetchBasis.hs:50-59)


def _shell_order(atoms):
    """The same functions with each d shell's components in createCGF order
    (the direct J/K kernels group complete shells in that order; the SCF energy
    does not depend on the order of the basis functions)."""
    out = []
    for a in atoms:
        cg = list(a.basis)
        ds = [c for c in cg if c.funtype.startswith("D")]
        if ds:
            rest = [c for c in cg if not c.funtype.startswith("D")]
            cg = rest + sorted(ds, key=lambda c: D_ORDER.index(c.funtype))
        out.append(B.AtomData(a.coord, cg, a.znumber, a.label))
    return out


@pytest.mark.parametrize("name", sorted(SAMPLES))
def test_sample_project_exact_mode(ctx, name):
    rec = SAMPLES[name]
    atoms = sample_atoms(rec)
    fb = B.flatten(_shell_order(atoms))
    ctx.set_basis(fb)
    r = ctx.scf(_lib.baseline_opts(charge=rec["charge"]), want_matrices=False)
    assert abs(r["energy"] - rec["oracle_energy_exact"]) < 1e-8
    rm = ctx.scf(_lib.baseline_opts(charge=rec["charge"], precision=_lib.PREC_MIXED, incremental=1),
                 want_matrices=False)
    assert abs(rm["energy"] - rec["oracle_energy_exact"]) < 1e-6


@pytest.mark.parametrize("name", sorted(SAMPLES))
def test_sample_project_reference_mode(ctx, name):
    """The reference's numerics and driver on the literal inputs in their own
    function order; the 6-31G* project's Harris guess leaves the ERI array."""
    rec = SAMPLES[name]
    fb = B.flatten(sample_atoms(rec))
    ctx.set_basis(fb)
    ctx.generate_boys_grid()
    opts = _lib.reference_opts(charge=rec["charge"])
    if rec["oracle_energy_reference"] is None:
        with pytest.raises(_lib.GBHFError) as e:
            ctx.scf(opts)
        assert e.value.name == "GBHF_ERR_INDEX"
        return
    r = ctx.scf(opts)
    assert abs(r["energy"] - rec["oracle_energy_reference"]) < 1e-8
    o = O.scf(fb, O.SCFOptions(charge=rec["charge"]))
    assert r["iterations"] == o.iterations
