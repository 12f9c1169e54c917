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

Three s/p classes run a second form in the J/K kernels ((ps|ps), and (pp|ss),
(pp|ps) with the lower pair as the warp-shared bra): per primitive quartet the
bra Hermite functions are contracted onto the ket's Hermite indices,
V[ab][h] += sum_tuv E^ab_tuv R_(tuv+h), and the ket transformation runs once
per ket primitive and bra-primitive range.  ``F_KERNEL`` counts, for those
classes, the work per primitive quartet of that form (R recursion, Boys values,
bra E products, the V contraction) and leaves out the per-ket-primitive
transformation: a lower bound of the work the kernel does, used for the
roofline of the J/K kernels.  For every other class F_KERNEL = F_alg.
"""
from math import comb

CLASSES = {"ssss": (0, 0, 0, 0), "psss": (1, 0, 0, 0), "psps": (1, 0, 1, 0),
           "ppss": (1, 1, 0, 0), "ppps": (1, 1, 1, 0), "pppp": (1, 1, 1, 1),
           "dsss": (2, 0, 0, 0), "dsps": (2, 0, 1, 0), "dspp": (2, 0, 1, 1), "dsds": (2, 0, 2, 0),
           "dpss": (2, 1, 0, 0), "dpps": (2, 1, 1, 0), "dppp": (2, 1, 1, 1), "dpds": (2, 1, 2, 0),
           "dpdp": (2, 1, 2, 1), "ddss": (2, 2, 0, 0), "ddps": (2, 2, 1, 0), "ddpp": (2, 2, 1, 1),
           "ddds": (2, 2, 2, 0), "dddp": (2, 2, 2, 1), "dddd": (2, 2, 2, 2)}

# classes in the deferred form: (warp-shared bra pair, per-lane ket pair)
DEFERRED = {"psps": ((1, 0), (1, 0)), "ppss": ((0, 0), (1, 1)), "ppps": ((1, 0), (1, 1))}


def ncart(l):
    return (l + 1) * (l + 2) // 2


def _cart(l):
    return [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]


def _hermite(a, b):
    return [(t, u, v) for t in range(a[0] + b[0] + 1) for u in range(a[1] + b[1] + 1) for v in range(a[2] + b[2] + 1)]


def flops_per_prim_quartet(la, lb, lc, ld):
    L = la + lb + lc + ld
    h_ab, h_cd = comb(la + lb + 3, 3), comb(lc + ld + 3, 3)
    n_ab, n_cd = ncart(la) * ncart(lb), ncart(lc) * ncart(ld)
    return (2 * comb(L + 4, 4) + 2 * h_ab * h_cd * n_cd + 2 * h_ab * n_ab * n_cd + 2 * n_ab * n_cd
            + 25 * (L + 1))


def flops_per_prim_quartet_deferred(bra, ket):
    """Work per primitive quartet of the deferred form (bra = warp-shared pair)."""
    (la, lb), (lc, ld) = bra, ket
    L = la + lb + lc + ld
    bra_terms = sum(len(_hermite(a, b)) for a in _cart(la) for b in _cart(lb))
    ket_union = {h for c in _cart(lc) for d in _cart(ld) for h in _hermite(c, d)}
    return 2 * comb(L + 4, 4) + 25 * (L + 1) + 2 * bra_terms + 2 * bra_terms * len(ket_union)


F_ALG = {name: flops_per_prim_quartet(*ls) for name, ls in CLASSES.items()}
F_KERNEL = {name: (flops_per_prim_quartet_deferred(*DEFERRED[name]) if name in DEFERRED else f)
            for name, f in F_ALG.items()}
