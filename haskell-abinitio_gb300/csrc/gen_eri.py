"""Emit straight-line McMurchie-Davidson primitive-quartet code per ERI class.

For a shell-quartet class (la lb | lc ld) this writes a device function that,
for one ket primitive pair held in registers, loops over the bra primitive
pairs staged in shared memory and accumulates every Cartesian component
integral (ab|cd) into an accumulator object.  The arithmetic follows the
McMurchie-Davidson scheme used by the reference
(Integrals/IntegralsEvaluation.hs:340-477):

    (ab|cd) = pref * sum_tuv E^ab_tuv sum_(tau nu phi) (-1)^(tau+nu+phi)
                     E^cd_(tau nu phi) R_(t+tau, u+nu, v+phi)(alpha, P-Q)

with the Hermite expansion coefficients from the same recursion as
``recursiveHermCoeff`` (t = 0: X_PA E^(i-1,j)_0 + E^(i-1,j)_1, ...; t >= 1:
(i E^(i-1,j)_(t-1) + j E^(i,j-1)_(t-1)) / (2 p t)) and R from the recursion
of ``calcHermM`` (reduce t first, then u, then v).  The prefactor
2 pi^(5/2) / (p q sqrt(p+q)) and both contraction products are folded into
R^(n)_000 = pref (-2 alpha)^n F_n(T), so the inner code is pure FMAs.

The generated file is ``eri_gen.cuh``; run ``python gen_eri.py`` after editing.
"""
from itertools import product
from pathlib import Path

CART = {0: [(0, 0, 0)], 1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
        2: [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)]}
LNAME = "spd"


def e_axis_code(prefix, pa, pb, h, lmax_a, lmax_b, needed):
    """Code computing E^(i,j)_t for one axis (E^00_0 = 1; the Gaussian factor is in K).

    ``needed`` is a set of (i, j, t); returns (lines, name map).  Zero terms
    are omitted (name None).
    """
    memo = {}
    lines = []

    def name(i, j, t):
        if i < 0 or j < 0 or t < 0 or t > i + j:
            return None
        key = (i, j, t)
        if key in memo:
            return memo[key]
        if i == 0 and j == 0 and t == 0:
            memo[key] = "ONE"
            return "ONE"
        if t == 0 and i >= 1:
            a, b = name(i - 1, j, 0), name(i - 1, j, 1)
            terms = []
            if a is not None:
                terms.append(pa if a == "ONE" else f"{pa} * {a}")
            if b is not None:
                terms.append(b)
        elif t == 0:
            a, b = name(i, j - 1, 0), name(i, j - 1, 1)
            terms = []
            if a is not None:
                terms.append(pb if a == "ONE" else f"{pb} * {a}")
            if b is not None:
                terms.append(b)
        else:
            a, b = name(i - 1, j, t - 1), name(i, j - 1, t - 1)
            inner = []
            if a is not None:
                inner.append(a if i == 1 else f"T({i}) * {a}")
            if b is not None:
                inner.append(b if j == 1 else f"T({j}) * {b}")
            if not inner:
                memo[key] = None
                return None
            s = " + ".join(inner)
            coef = h if t == 1 else f"({h} * T({1.0 / t!r}))"
            terms = [f"{coef} * ({s})"]
        if not terms:
            memo[key] = None
            return None
        nm = f"{prefix}{i}{j}{t}"
        lines.append(f"const T {nm} = {' + '.join(terms)};")
        memo[key] = nm
        return nm

    for (i, j, t) in sorted(needed):
        name(i, j, t)
    return lines, memo


def r_code(L, needed):
    """Code computing R^0_tuv (scaled) for all (t,u,v) in ``needed``."""
    memo = {}
    lines = []

    def name(n, t, u, v):
        if t < 0 or u < 0 or v < 0:
            return None
        key = (n, t, u, v)
        if key in memo:
            return memo[key]
        if t == 0 and u == 0 and v == 0:
            nm = f"R{n}_000"
            memo[key] = nm
            return nm
        if t >= 1:
            a, b, x, k = name(n + 1, t - 2, u, v), name(n + 1, t - 1, u, v), "X", t - 1
        elif u >= 1:
            a, b, x, k = name(n + 1, t, u - 2, v), name(n + 1, t, u - 1, v), "Y", u - 1
        else:
            a, b, x, k = name(n + 1, t, u, v - 2), name(n + 1, t, u, v - 1), "Z", v - 1
        terms = []
        if a is not None and k != 0:
            terms.append(a if k == 1 else f"T({k}) * {a}")
        if b is not None:
            terms.append(f"{x} * {b}")
        nm = f"R{n}_{t}{u}{v}"
        lines.append(f"const T {nm} = {' + '.join(terms)};")
        memo[key] = nm
        return nm

    for (t, u, v) in sorted(needed, key=lambda k: (sum(k), k)):
        name(0, t, u, v)
    used_n = sorted({k[0] for k in memo if k[1:] == (0, 0, 0)})
    return lines, memo, used_n


def gen_class(la, lb, lc, ld):
    ca, cb, cc, cd = CART[la], CART[lb], CART[lc], CART[ld]
    L = la + lb + lc + ld
    nab, ncd = len(ca) * len(cb), len(cc) * len(cd)
    cls = f"{LNAME[la]}{LNAME[lb]}{LNAME[lc]}{LNAME[ld]}"
    # Hermite index sets
    bra_h = {}   # ab -> list of (t,u,v)
    for ia, a in enumerate(ca):
        for ib, b in enumerate(cb):
            bra_h[(ia, ib)] = [(t, u, v) for t in range(a[0] + b[0] + 1)
                               for u in range(a[1] + b[1] + 1) for v in range(a[2] + b[2] + 1)]
    ket_h = {}
    for ic, c in enumerate(cc):
        for idd, d in enumerate(cd):
            ket_h[(ic, idd)] = [(t, u, v) for t in range(c[0] + d[0] + 1)
                                for u in range(c[1] + d[1] + 1) for v in range(c[2] + d[2] + 1)]
    bra_union = sorted({h for hs in bra_h.values() for h in hs}, key=lambda k: (sum(k), k))
    needed_r = set()
    for hs in ket_h.values():
        for (tk, uk, vk) in hs:
            for (tb, ub, vb) in bra_union:
                needed_r.add((tb + tk, ub + uk, vb + vk))
    r_lines, r_memo, used_n = r_code(L, needed_r)

    # per-axis E needs
    def axis_needs(cs_a, cs_b):
        need = [set(), set(), set()]
        for a in cs_a:
            for b in cs_b:
                for x in range(3):
                    for t in range(a[x] + b[x] + 1):
                        need[x].add((a[x], b[x], t))
        return need

    out = []
    w = out.append
    w(f"// ---- class ({cls[0]}{cls[1]}|{cls[2]}{cls[3]}): {nab}x{ncd} integrals, L = {L}")
    w("template <typename T, typename Acc>")
    w(f"__device__ __forceinline__ void eri_ketprim_{cls}(const T* __restrict__ sb, int nbra, int bstep,")
    w("    const T q, const T invq, const T Qx, const T Qy, const T Qz,")
    w("    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,")
    w("    const T Kcd, const T* __restrict__ boys, Acc& acc) {")
    w("  const T ONE = T(1);")
    w("  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;")
    # ket E (hoisted out of the bra loop)
    w("  const T hq = T(0.5) * invq;")
    kneed = axis_needs(cc, cd)
    kmaps = []
    for x, ax in enumerate("xyz"):
        lines, memo = e_axis_code(f"ek{ax}", f"QC{ax}", f"QD{ax}", "hq", lc, ld, kneed[x])
        for ln in lines:
            w("  " + ln)
        kmaps.append(memo)
    # ket E products with sign: ekp_<cd>_<tuv>
    ket_terms = {}
    for (ic, idd), hs in ket_h.items():
        c, d = cc[ic], cd[idd]
        lst = []
        for (t, u, v) in hs:
            fx = kmaps[0].get((c[0], d[0], t))
            fy = kmaps[1].get((c[1], d[1], u))
            fz = kmaps[2].get((c[2], d[2], v))
            if fx is None or fy is None or fz is None:
                continue
            fac = [f for f in (fx, fy, fz) if f != "ONE"]
            sign = -1 if (t + u + v) % 2 else 1
            nm = f"ekp{ic}{idd}_{t}{u}{v}"
            if not fac:
                expr = "ONE" if sign > 0 else "-ONE"
            else:
                expr = " * ".join(fac)
                if sign < 0:
                    expr = f"-({expr})"
            w(f"  const T {nm} = {expr};")
            lst.append((nm, (t, u, v)))
        ket_terms[(ic, idd)] = lst
    # (ss|ss) and (ps|ss): two bra primitives in flight (two independent load
    # and Boys chains; the larger classes keep their registers for one)
    w("  #pragma unroll 2" if L <= 1 else "  #pragma unroll 1")
    w("  for (int kb = 0; kb < nbra; ++kb) {")
    w("    BraPrim<T> bp;")
    w("    load_bra_prim(sb + kb * bstep, bp);")
    w("    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;")
    if la >= 1:
        w("    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;")
    if lb >= 1:
        w("    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;")
    w("    const T Kab = bp.K;")
    w("    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;")
    w("    const T ppq = p + q;")
    w("    const T rs = rsqrt_t(ppq);")
    w("    const T alpha = p * q * (rs * rs);")
    w("    const T Tb = alpha * (X * X + Y * Y + Z * Z);")
    w("    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p")
    w(f"    T F[{L + 1}];")
    w(f"    boys_eval<T, {L}>(Tb, boys, F);")
    w("    const T m2a = T(-2) * alpha;")
    w("    T scale = pref;")
    for n in range(L + 1):
        if n in used_n:
            w(f"    const T R{n}_000 = scale * F[{n}];")
        if n < L:
            w("    scale *= m2a;")
    for ln in r_lines:
        w("    " + ln)
    # bra E
    w("    const T hp = T(0.5) * invp;")
    bneed = axis_needs(ca, cb)
    bmaps = []
    for x, ax in enumerate("xyz"):
        lines, memo = e_axis_code(f"eb{ax}", f"PA{ax}", f"PB{ax}", "hp", la, lb, bneed[x])
        for ln in lines:
            w("    " + ln)
        bmaps.append(memo)
    bra_terms = {}
    for (ia, ib), hs in bra_h.items():
        a, b = ca[ia], cb[ib]
        lst = []
        for (t, u, v) in hs:
            fx = bmaps[0].get((a[0], b[0], t))
            fy = bmaps[1].get((a[1], b[1], u))
            fz = bmaps[2].get((a[2], b[2], v))
            if fx is None or fy is None or fz is None:
                continue
            fac = [f for f in (fx, fy, fz) if f != "ONE"]
            lst.append((fac, (t, u, v)))
        bra_terms[(ia, ib)] = lst
    # per ket comp pair: W then accumulate into every bra comp pair
    for (ic, idd), kts in ket_terms.items():
        icd = ic * len(cd) + idd
        used_bh = sorted({h for lst in bra_terms.values() for (_, h) in lst}, key=lambda k: (sum(k), k))
        w("    {")
        for (tb, ub, vb) in used_bh:
            terms = []
            for (nm, (tk, uk, vk)) in kts:
                r = r_memo[(0, tb + tk, ub + uk, vb + vk)]
                terms.append((nm, r))
            expr = None
            for nm, r in terms:
                if expr is None:
                    expr = f"{r}" if nm == "ONE" else (f"-{r}" if nm == "-ONE" else f"{nm} * {r}")
                else:
                    if nm == "ONE":
                        expr = f"{expr} + {r}"
                    elif nm == "-ONE":
                        expr = f"{expr} - {r}"
                    else:
                        expr = f"fma_t({nm}, {r}, {expr})"
            w(f"      const T W_{tb}{ub}{vb} = {expr};")
        for (ia, ib), lst in bra_terms.items():
            iab = ia * len(cb) + ib
            idx = iab * ncd + icd
            expr = None
            for fac, (t, u, v) in lst:
                wn = f"W_{t}{u}{v}"
                coef = " * ".join(fac) if fac else None
                if expr is None:
                    expr = wn if coef is None else f"{coef} * {wn}"
                else:
                    expr = f"{expr} + {wn}" if coef is None else f"fma_t({coef}, {wn}, {expr})"
            w(f"      acc[{idx}] += {expr};")
        w("    }")
    w("  }")
    w("}")
    return "\n".join(out), cls, nab, ncd, L


def gen_class_deferred(la, lb, lc, ld):
    """The same integrals with the ket (per-lane) transformation deferred.

    For one ket primitive the bra loop accumulates
        V[ab][h] = sum_bra sum_tuv E^ab_tuv R_(tuv + h)      (h: ket Hermite indices)
    and the ket coefficients (sign included) act once after the loop:
        acc[ab][cd] += sum_h (-1)^|h| E^cd_h V[ab][h].
    Per primitive quartet this leaves the R recursion and the bra transformation
    onto the ket Hermite indices; the ket transformation, the larger one when the
    per-lane pair carries the higher angular momentum, is paid once per ket
    primitive and bra-primitive range.  Used with the lower-momentum pair as the
    warp-shared bra.
    """
    ca, cb, cc, cd = CART[la], CART[lb], CART[lc], CART[ld]
    L = la + lb + lc + ld
    nab, ncd = len(ca) * len(cb), len(cc) * len(cd)
    cls = f"{LNAME[la]}{LNAME[lb]}{LNAME[lc]}{LNAME[ld]}"
    bra_h = {}
    for ia, a in enumerate(ca):
        for ib, b in enumerate(cb):
            bra_h[(ia, ib)] = [(t, u, v) for t in range(a[0] + b[0] + 1)
                               for u in range(a[1] + b[1] + 1) for v in range(a[2] + b[2] + 1)]
    ket_h = {}
    for ic, c in enumerate(cc):
        for idd, d in enumerate(cd):
            ket_h[(ic, idd)] = [(t, u, v) for t in range(c[0] + d[0] + 1)
                                for u in range(c[1] + d[1] + 1) for v in range(c[2] + d[2] + 1)]

    def axis_needs(cs_a, cs_b):
        need = [set(), set(), set()]
        for a in cs_a:
            for b in cs_b:
                for x in range(3):
                    for t in range(a[x] + b[x] + 1):
                        need[x].add((a[x], b[x], t))
        return need

    out = []
    w = out.append
    w(f"// ---- class ({cls[0]}{cls[1]}|{cls[2]}{cls[3]}): {nab}x{ncd} integrals, L = {L}, ket transformation deferred")
    w("template <typename T, typename Acc>")
    w(f"__device__ __forceinline__ void eri_ketprim_{cls}(const T* __restrict__ sb, int nbra, int bstep,")
    w("    const T q, const T invq, const T Qx, const T Qy, const T Qz,")
    w("    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,")
    w("    const T Kcd, const T* __restrict__ boys, Acc& acc) {")
    w("  const T ONE = T(1);")
    w("  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;")
    w("  const T hq = T(0.5) * invq;")
    kneed = axis_needs(cc, cd)
    kmaps = []
    for x, ax in enumerate("xyz"):
        lines, memo = e_axis_code(f"ek{ax}", f"QC{ax}", f"QD{ax}", "hq", lc, ld, kneed[x])
        for ln in lines:
            w("  " + ln)
        kmaps.append(memo)
    ket_terms = {}
    for (ic, idd), hs in ket_h.items():
        c, d = cc[ic], cd[idd]
        lst = []
        for (t, u, v) in hs:
            fx = kmaps[0].get((c[0], d[0], t))
            fy = kmaps[1].get((c[1], d[1], u))
            fz = kmaps[2].get((c[2], d[2], v))
            if fx is None or fy is None or fz is None:
                continue
            fac = [f for f in (fx, fy, fz) if f != "ONE"]
            sign = -1 if (t + u + v) % 2 else 1
            nm = f"ekp{ic}{idd}_{t}{u}{v}"
            if not fac:
                expr = "ONE" if sign > 0 else "-ONE"
            else:
                expr = " * ".join(fac)
                if sign < 0:
                    expr = f"-({expr})"
            w(f"  const T {nm} = {expr};")
            lst.append((nm, (t, u, v)))
        ket_terms[(ic, idd)] = lst
    ket_union = sorted({h for lst in ket_terms.values() for (_, h) in lst}, key=lambda k: (sum(k), k))
    # bra E (per bra primitive)
    bneed = axis_needs(ca, cb)
    bra_union = sorted({h for hs in bra_h.values() for h in hs}, key=lambda k: (sum(k), k))
    needed_r = set()
    for (tk, uk, vk) in ket_union:
        for (tb, ub, vb) in bra_union:
            needed_r.add((tb + tk, ub + uk, vb + vk))
    r_lines, r_memo, used_n = r_code(L, needed_r)
    for iab in range(nab):
        for h in ket_union:
            w(f"  T V{iab}_{h[0]}{h[1]}{h[2]} = T(0);")
    w("  #pragma unroll 1")
    w("  for (int kb = 0; kb < nbra; ++kb) {")
    w("    BraPrim<T> bp;")
    w("    load_bra_prim(sb + kb * bstep, bp);")
    w("    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;")
    if la >= 1:
        w("    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;")
    if lb >= 1:
        w("    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;")
    w("    const T Kab = bp.K;")
    w("    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;")
    w("    const T ppq = p + q;")
    w("    const T rs = rsqrt_t(ppq);")
    w("    const T alpha = p * q * (rs * rs);")
    w("    const T Tb = alpha * (X * X + Y * Y + Z * Z);")
    w("    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p")
    w(f"    T F[{L + 1}];")
    w(f"    boys_eval<T, {L}>(Tb, boys, F);")
    w("    const T m2a = T(-2) * alpha;")
    w("    T scale = pref;")
    for n in range(L + 1):
        if n in used_n:
            w(f"    const T R{n}_000 = scale * F[{n}];")
        if n < L:
            w("    scale *= m2a;")
    for ln in r_lines:
        w("    " + ln)
    if la + lb > 0:
        w("    const T hp = T(0.5) * invp;")
    else:
        w("    (void)invp;")
    bmaps = []
    for x, ax in enumerate("xyz"):
        lines, memo = e_axis_code(f"eb{ax}", f"PA{ax}", f"PB{ax}", "hp", la, lb, bneed[x])
        for ln in lines:
            w("    " + ln)
        bmaps.append(memo)
    for (ia, ib), hs in bra_h.items():
        a, b = ca[ia], cb[ib]
        iab = ia * len(cb) + ib
        lst = []
        for (t, u, v) in hs:
            fx = bmaps[0].get((a[0], b[0], t))
            fy = bmaps[1].get((a[1], b[1], u))
            fz = bmaps[2].get((a[2], b[2], v))
            if fx is None or fy is None or fz is None:
                continue
            fac = [f for f in (fx, fy, fz) if f != "ONE"]
            lst.append((fac, (t, u, v)))
        for h in ket_union:
            vn = f"V{iab}_{h[0]}{h[1]}{h[2]}"
            expr = vn
            for fac, (t, u, v) in lst:
                r = r_memo[(0, t + h[0], u + h[1], v + h[2])]
                coef = " * ".join(fac) if fac else None
                expr = f"{expr} + {r}" if coef is None else f"fma_t({coef}, {r}, {expr})"
            w(f"    {vn} = {expr};")
    w("  }")
    for iab in range(nab):
        for (ic, idd), kts in ket_terms.items():
            icd = ic * len(cd) + idd
            expr = None
            for nm, h in kts:
                vn = f"V{iab}_{h[0]}{h[1]}{h[2]}"
                if expr is None:
                    expr = vn if nm == "ONE" else (f"-{vn}" if nm == "-ONE" else f"{nm} * {vn}")
                elif nm == "ONE":
                    expr = f"{expr} + {vn}"
                elif nm == "-ONE":
                    expr = f"{expr} - {vn}"
                else:
                    expr = f"fma_t({nm}, {vn}, {expr})"
            w(f"  acc[{iab * ncd + icd}] += {expr};")
    w("}")
    return "\n".join(out), cls, nab, ncd, L


def render():
    """The text of eri_gen.cuh."""
    # s/p classes: (ss|ss), (ps|ss) and (pp|pp) as they are; (ps|ps), and (pp|ss)
    # and (pp|ps) with the lower pair as the warp-shared bra, with the ket
    # transformation deferred.  For (ps|ss) the swapped form saved FP64 time but
    # lost more in FP32, where the extra tasks of the ss-pair bras cost more than
    # the small bra transformation it saves.
    classes = [(0, 0, 0, 0), (1, 0, 0, 0), (1, 1, 1, 1)]
    deferred = [(1, 0, 1, 0), (0, 0, 1, 1), (1, 0, 1, 1)]
    # the d classes with few components per quartet (the larger ones use the
    # warp-per-quartet kernels of jkd.cu)
    classes += [(2, 0, 0, 0), (2, 0, 1, 0), (2, 0, 1, 1), (2, 0, 2, 0), (2, 1, 0, 0), (2, 1, 1, 0), (2, 2, 0, 0)]
    parts = ["// GENERATED by gen_eri.py -- do not edit by hand.",
             "#pragma once", ""]
    for c in classes:
        code, *_ = gen_class(*c)
        parts.append(code)
        parts.append("")
    for c in deferred:
        code, *_ = gen_class_deferred(*c)
        parts.append(code)
        parts.append("")
    return "\n".join(parts)


def main():
    Path(__file__).with_name("eri_gen.cuh").write_text(render())


if __name__ == "__main__":
    main()
