"""Algorithmic FLOP model of one primitive shell quartet (McMurchie-Davidson).

For a class (la lb | lc ld) with L = la+lb+lc+ld, n_x Cartesian components
and H_ab = C(la+lb+3, 3) bra Hermite functions:

    F_alg = 2 C(L+4, 4)            R^n_tuv recursion
          + 2 H_ab H_cd n_cd       ket Hermite contraction
          + 2 H_ab n_ab n_cd       bra contraction
          + 2 n_ab n_cd            accumulation over primitives
          + 25 (L+1)               Boys function values

giving 33, 98, 291, 323, 1004, 3847 flops for (ss|ss) ... (pp|pp).  The same
model is applied to the GPU kernels and to the CPU oracle, so the numbers
compare work, not implementation details.
"""
from math import comb

CLASSES = {"ssss": (0, 0, 0, 0), "psss": (1, 0, 0, 0), "psps": (1, 0, 1, 0),
           "ppss": (1, 1, 0, 0), "ppps": (1, 1, 1, 0), "pppp": (1, 1, 1, 1)}


def ncart(l):
    return (l + 1) * (l + 2) // 2


def flops_per_prim_quartet(la, lb, lc, ld):
    L = la + lb + lc + ld
    h_ab, h_cd = comb(la + lb + 3, 3), comb(lc + ld + 3, 3)
    n_ab, n_cd = ncart(la) * ncart(lb), ncart(lc) * ncart(ld)
    return (2 * comb(L + 4, 4) + 2 * h_ab * h_cd * n_cd + 2 * h_ab * n_ab * n_cd + 2 * n_ab * n_cd
            + 25 * (L + 1))


F_ALG = {name: flops_per_prim_quartet(*ls) for name, ls in CLASSES.items()}
