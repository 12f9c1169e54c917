"""The oracle's superposition-of-atomic-densities guess (a library feature
with no reference counterpart): electron count, spherical atoms, block
structure."""
import numpy as np

import oracle as O
from gbhf import basis as B, molecules as M


def test_atomic_density_oxygen_631g():
    fb = B.flatten(M.water_atoms("6-31g", "text"))
    sub, idx = O._atom_sub_basis(fb, 0)
    d = O.atomic_density(sub)
    s = O.tri_to_square(O.OracleBasis(sub).overlap(False))
    assert abs(np.trace(d @ s) - 8.0) < 1e-10
    np.testing.assert_allclose(d, d.T, atol=1e-13)
    # spherical: the three p components carry the same population
    pop = np.diag(d @ s)
    lx = sub.cgf_lxyz
    for shell in (idx[lx.sum(axis=1) == 1].reshape(-1, 3) - idx[0]):
        assert np.ptp(pop[shell]) < 1e-10


def test_fractional_occupations():
    eps = np.array([-20.0, -1.2, -0.4, -0.4 + 1e-9, -0.4 - 1e-9, 1.1])
    np.testing.assert_allclose(O.fractional_occupations(eps, 8.0), [2, 2, 4 / 3, 4 / 3, 4 / 3, 0])
    np.testing.assert_allclose(O.fractional_occupations(np.array([-0.2, 0.9]), 1.0), [1, 0])


def test_sad_density_cluster():
    fb = B.flatten(M.cluster_atoms("batch256", "sto-3g", index=20))
    d = O.tri_to_square(O.sad_density(fb))
    s = O.tri_to_square(O.OracleBasis(fb).overlap(False))
    assert abs(np.trace(d @ s) - fb.charge.sum()) < 1e-9
    same = fb.cgf_atom[:, None] == fb.cgf_atom[None, :]
    assert np.all(d[~same] == 0.0)
