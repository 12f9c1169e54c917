"""Emit straight-line McMurchie-Davidson code for the two-electron gradient.

For a shell-quartet class (la lb | lc ld) this writes a device function that,
for one ket primitive pair in registers, loops over the bra primitive pairs
staged in shared memory and accumulates the bra-centre derivatives

    g_A,x += sum_abcd Gamma_abcd d(ab|cd)/dA_x,    g_B,x likewise,

with the derivative of a Cartesian Gaussian taken on the basis function,
d/dA_x [x_A^i exp(-a r_A^2)] = 2a x_A^(i+1) exp(..) - i x_A^(i-1) exp(..)
(the relation the reference's calcDervCGF uses, HartreeFock/Derivatives.hs:
246-257), so that in Hermite form the x factor E^(i,j)_t of the bra is
replaced by 2a E^(i+1,j)_t - i E^(i-1,j)_t.  The Gaussian-product factor
K_ab is part of every E^(i,j) alike, so no separate derivative of K appears.

The ket side is contracted with Gamma first, per bra component pair ab:

    T_ab(tau nu phi) = sum_cd Gamma_abcd (-1)^(tau+nu+phi) E^cd_(tau nu phi)
    U_ab(t u v)      = sum_(tau nu phi) T_ab(tau nu phi) R_(t+tau, u+nu, v+phi)
    g_A,x           += sum_tuv [2a E^(i+1,j)_t - i E^(i-1,j)_t] E_u E_v U_ab(tuv)

with R up to order L + 1 and the prefactor folded into R^(n)_000 as in
gen_eri.py.  The generated file is ``grad_gen.cuh``; run
``python gen_grad.py`` after editing.
"""
from pathlib import Path

from gen_eri import CART, LNAME, e_axis_code, r_code


def gen_class(la, lb, lc, ld):
    ca, cb, cc, cd = CART[la], CART[lb], CART[lc], CART[ld]
    L = la + lb + lc + ld + 1
    ncd = len(cc) * len(cd)
    cls = f"{LNAME[la]}{LNAME[lb]}{LNAME[lc]}{LNAME[ld]}"
    # ket Hermite terms per cd (signed products, hoisted out of the bra loop)
    ket_h = {}
    for ic, c in enumerate(cc):
        for idd, d in enumerate(cd):
            ket_h[(ic, idd)] = [(t, u, v) for t in range(c[0] + d[0] + 1)
                                for u in range(c[1] + d[1] + 1) for v in range(c[2] + d[2] + 1)]
    ket_union = sorted({h for hs in ket_h.values() for h in hs}, key=lambda k: (sum(k), k))

    # bra: per ab, the Hermite indices each derivative needs
    def dsets(a, b):
        """{(side, dir): [(t,u,v)]} for side in 'AB', dir in 0..2."""
        out = {}
        for side in "AB":
            for d in range(3):
                rng = [a[x] + b[x] + (1 if x == d else 0) for x in range(3)]
                out[(side, d)] = [(t, u, v) for t in range(rng[0] + 1) for u in range(rng[1] + 1)
                                  for v in range(rng[2] + 1)]
        return out

    bra = {}
    for ia, a in enumerate(ca):
        for ib, b in enumerate(cb):
            ds = dsets(a, b)
            uset = sorted({h for hs in ds.values() for h in hs}, key=lambda k: (sum(k), k))
            bra[(ia, ib)] = (a, b, ds, uset)
    needed_r = set()
    for (_, _, _, uset) in bra.values():
        for (tb, ub, vb) in uset:
            for (tk, uk, vk) in ket_union:
                needed_r.add((tb + tk, ub + uk, vb + vk))
    r_lines, r_memo, used_n = r_code(L, needed_r)

    # E needs per axis (bra): (i, j, t) incl. i+1 / j+1 / i-1 / j-1
    bneed = [set(), set(), set()]
    for (a, b, _, _) in bra.values():
        for x in range(3):
            i, j = a[x], b[x]
            for t in range(i + j + 1):
                bneed[x].add((i, j, t))
            for t in range(i + j + 2):
                bneed[x].add((i + 1, j, t))
                bneed[x].add((i, j + 1, t))
            if i >= 1:
                for t in range(i + j):
                    bneed[x].add((i - 1, j, t))
            if j >= 1:
                for t in range(i + j):
                    bneed[x].add((i, j - 1, t))
    kneed = [set(), set(), set()]
    for c in cc:
        for d in cd:
            for x in range(3):
                for t in range(c[x] + d[x] + 1):
                    kneed[x].add((c[x], d[x], t))

    out = []
    w = out.append
    w(f"// ---- gradient class ({cls[0]}{cls[1]}|{cls[2]}{cls[3]}): bra-centre derivatives, L + 1 = {L}")
    w("template <typename T, typename G>")
    w(f"__device__ __forceinline__ void grad_ketprim_{cls}(const T* __restrict__ sb, int nbra, int bstep,")
    w("    const T q, const T invq, const T Qx, const T Qy, const T Qz,")
    w("    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,")
    w("    const T Kcd, const T* __restrict__ boys, const G& gam, T* g) {")
    w("  const T ONE = T(1);")
    w("  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;")
    w("  const T hq = T(0.5) * invq;")
    kmaps = []
    for x, ax in enumerate("xyz"):
        lines, memo = e_axis_code(f"ek{ax}", f"QC{ax}", f"QD{ax}", "hq", lc, ld, kneed[x])
        for ln in lines:
            w("  " + ln)
        kmaps.append(memo)
    ket_terms = {}
    for (ic, idd), hs in ket_h.items():
        c, d = cc[ic], cd[idd]
        lst = {}
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
            lst[(t, u, v)] = nm
        ket_terms[(ic, idd)] = lst
    w("  #pragma unroll 1")
    w("  for (int kb = 0; kb < nbra; ++kb) {")
    w("    BraPrim<T> bp;")
    w("    load_bra_prim(sb + kb * bstep, bp);")
    w("    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;")
    w("    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;")
    w("    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;")
    w("    const T Kab = bp.K;")
    w("    const T ea = bp.a;")
    w("    const T ta = T(2) * ea, tb = T(2) * (p - ea);")
    w("    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;")
    w("    const T ppq = p + q;")
    w("    const T rs = rsqrt_t(ppq);")
    w("    const T alpha = p * q * (rs * rs);")
    w("    const T Tb = alpha * (X * X + Y * Y + Z * Z);")
    w("    const T pref = Kab * Kcd * rs;")
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
    w("    const T hp = T(0.5) * invp;")
    bmaps = []
    for x, ax in enumerate("xyz"):
        lines, memo = e_axis_code(f"eb{ax}", f"PA{ax}", f"PB{ax}", "hp", la + 1, lb + 1, bneed[x])
        for ln in lines:
            w("    " + ln)
        bmaps.append(memo)

    # derivative factors per axis: dA(i,j,t) = ta E(i+1,j,t) - i E(i-1,j,t); dB likewise
    dnames = {}

    def dfac(side, x, i, j, t):
        key = (side, x, i, j, t)
        if key in dnames:
            return dnames[key]
        m = bmaps[x]
        if side == "A":
            up, dn, k, tw = m.get((i + 1, j, t)), (m.get((i - 1, j, t)) if i >= 1 else None), i, "ta"
        else:
            up, dn, k, tw = m.get((i, j + 1, t)), (m.get((i, j - 1, t)) if j >= 1 else None), j, "tb"
        terms = []
        if up is not None:
            terms.append(tw if up == "ONE" else f"{tw} * {up}")
        if dn is not None:
            c = "" if k == 1 else f"T({k}) * "
            terms.append(f"- {c}{'ONE' if dn == 'ONE' else dn}")
        if not terms:
            dnames[key] = None
            return None
        nm = f"d{side}{'xyz'[x]}{i}{j}_{t}"
        expr = terms[0] + (" " + terms[1] if len(terms) > 1 else "")
        w(f"    const T {nm} = {expr};")
        dnames[key] = nm
        return nm

    # declare every derivative factor at loop scope (shared by the ab blocks)
    for (a, b, ds, _) in bra.values():
        for side in "AB":
            for d in range(3):
                for tt in ds[(side, d)]:
                    dfac(side, d, a[d], b[d], tt[d])

    for (ia, ib), (a, b, ds, uset) in bra.items():
        iab = ia * len(cb) + ib
        w("    {")
        # T_ab(tau) = sum_cd Gamma_abcd ekp_cd(tau)
        tnames = {}
        for tau in ket_union:
            expr = None
            for (ic, idd), lst in ket_terms.items():
                if tau not in lst:
                    continue
                icd = ic * len(cd) + idd
                gm = f"gam.get({iab * ncd + icd})"
                e = lst[tau]
                if e == "ONE":
                    term_add, term_fma = gm, None
                elif e == "-ONE":
                    term_add, term_fma = f"-{gm}", None
                else:
                    term_add, term_fma = None, (gm, e)
                if expr is None:
                    expr = term_add if term_add is not None else f"{term_fma[0]} * {term_fma[1]}"
                else:
                    expr = (f"{expr} + {term_add}" if term_add is not None
                            else f"fma_t({term_fma[0]}, {term_fma[1]}, {expr})")
            if expr is not None:
                nm = f"T_{tau[0]}{tau[1]}{tau[2]}"
                w(f"      const T {nm} = {expr};")
                tnames[tau] = nm
        # U_ab(tuv)
        unames = {}
        for (tb_, ub, vb) in uset:
            expr = None
            for tau, tn in tnames.items():
                r = r_memo[(0, tb_ + tau[0], ub + tau[1], vb + tau[2])]
                expr = f"{tn} * {r}" if expr is None else f"fma_t({tn}, {r}, {expr})"
            if expr is not None:
                nm = f"U_{tb_}{ub}{vb}"
                w(f"      const T {nm} = {expr};")
                unames[(tb_, ub, vb)] = nm
        # contractions
        for si, side in enumerate("AB"):
            for d in range(3):
                expr = None
                for (t, u, v) in ds[(side, d)]:
                    if (t, u, v) not in unames:
                        continue
                    tt = (t, u, v)
                    facs = []
                    ok = True
                    for x in range(3):
                        if x == d:
                            f = dfac(side, x, a[x], b[x], tt[x])
                        else:
                            f = bmaps[x].get((a[x], b[x], tt[x]))
                        if f is None:
                            ok = False
                            break
                        if f != "ONE":
                            facs.append(f)
                    if not ok:
                        continue
                    un = unames[tt]
                    coef = " * ".join(facs) if facs else None
                    if expr is None:
                        expr = un if coef is None else f"{coef} * {un}"
                    else:
                        expr = f"{expr} + {un}" if coef is None else f"fma_t({coef}, {un}, {expr})"
                if expr is not None:
                    w(f"      g[{3 * si + d}] += {expr};")
        w("    }")
    w("  }")
    w("}")
    return "\n".join(out), cls


def gen_vne(la, lb):
    """Nuclear-attraction derivatives of one primitive pair of class (la lb) for
    one nucleus C:  g_A,x += sum_ab w_ab dV^C_ab/dA_x,  g_B,x likewise, with
    V^C_ab = zpref sum_tuv E^ab_tuv R_tuv(p, P - C) (zpref = -Z_C 2 pi/p c_a c_b
    exp(-mu AB^2), w_ab the density weights) and the same derivative rule on
    the Hermite coefficients as the two-electron code.  The operator-centre
    derivative is -(g_A + g_B)."""
    ca, cb = CART[la], CART[lb]
    L = la + lb + 1
    cls = f"{LNAME[la]}{LNAME[lb]}"
    bra = {}
    for ia, a in enumerate(ca):
        for ib, b in enumerate(cb):
            ds = {}
            for side in "AB":
                for d in range(3):
                    rng = [a[x] + b[x] + (1 if x == d else 0) for x in range(3)]
                    ds[(side, d)] = [(t, u, v) for t in range(rng[0] + 1) for u in range(rng[1] + 1)
                                     for v in range(rng[2] + 1)]
            bra[(ia, ib)] = (a, b, ds)
    needed_r = {h for (_, _, ds) in bra.values() for hs in ds.values() for h in hs}
    r_lines, r_memo, used_n = r_code(L, needed_r)
    bneed = [set(), set(), set()]
    for (a, b, _) in bra.values():
        for x in range(3):
            i, j = a[x], b[x]
            for t in range(i + j + 1):
                bneed[x].add((i, j, t))
            for t in range(i + j + 2):
                bneed[x].add((i + 1, j, t))
                bneed[x].add((i, j + 1, t))
            if i >= 1:
                for t in range(i + j):
                    bneed[x].add((i - 1, j, t))
            if j >= 1:
                for t in range(i + j):
                    bneed[x].add((i, j - 1, t))
    out = []
    w = out.append
    w(f"// ---- nuclear-attraction gradient, pair class ({cls}): one primitive pair, one nucleus")
    w("template <typename T>")
    w(f"__device__ __forceinline__ void vne_grad_{cls}(const BraPrim<T>& bp, const T Cx, const T Cy, const T Cz,")
    w("    const T zpref, const T* __restrict__ dw, const T* __restrict__ boys, T* g) {")
    w("  const T ONE = T(1);")
    w("  const T p = bp.p, invp = bp.invp;")
    w("  const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz, PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;")
    w("  const T ta = T(2) * bp.a, tb = T(2) * (p - bp.a);")
    w("  const T X = bp.Px - Cx, Y = bp.Py - Cy, Z = bp.Pz - Cz;")
    w("  const T Tb = p * (X * X + Y * Y + Z * Z);")
    w(f"  T F[{L + 1}];")
    w(f"  boys_eval<T, {L}>(Tb, boys, F);")
    w("  const T m2a = T(-2) * p;")
    w("  T scale = zpref;")
    for n in range(L + 1):
        if n in used_n:
            w(f"  const T R{n}_000 = scale * F[{n}];")
        if n < L:
            w("  scale *= m2a;")
    for ln in r_lines:
        w("  " + ln)
    w("  const T hp = T(0.5) * invp;")
    bmaps = []
    for x, ax in enumerate("xyz"):
        lines, memo = e_axis_code(f"eb{ax}", f"PA{ax}", f"PB{ax}", "hp", la + 1, lb + 1, bneed[x])
        for ln in lines:
            w("  " + ln)
        bmaps.append(memo)
    dnames = {}

    def dfac(side, x, i, j, t):
        key = (side, x, i, j, t)
        if key in dnames:
            return dnames[key]
        m = bmaps[x]
        if side == "A":
            up, dn, k, tw = m.get((i + 1, j, t)), (m.get((i - 1, j, t)) if i >= 1 else None), i, "ta"
        else:
            up, dn, k, tw = m.get((i, j + 1, t)), (m.get((i, j - 1, t)) if j >= 1 else None), j, "tb"
        terms = []
        if up is not None:
            terms.append(tw if up == "ONE" else f"{tw} * {up}")
        if dn is not None:
            c = "" if k == 1 else f"T({k}) * "
            terms.append(f"- {c}{'ONE' if dn == 'ONE' else dn}")
        if not terms:
            dnames[key] = None
            return None
        nm = f"d{side}{'xyz'[x]}{i}{j}_{t}"
        w(f"  const T {nm} = {terms[0] + (' ' + terms[1] if len(terms) > 1 else '')};")
        dnames[key] = nm
        return nm

    for (a, b, ds) in bra.values():
        for side in "AB":
            for d in range(3):
                for tt in ds[(side, d)]:
                    dfac(side, d, a[d], b[d], tt[d])
    for (ia, ib), (a, b, ds) in bra.items():
        iab = ia * len(cb) + ib
        for si, side in enumerate("AB"):
            for d in range(3):
                expr = None
                for tt in ds[(side, d)]:
                    facs = []
                    ok = True
                    for x in range(3):
                        f = dfac(side, x, a[x], b[x], tt[x]) if x == d else bmaps[x].get((a[x], b[x], tt[x]))
                        if f is None:
                            ok = False
                            break
                        if f != "ONE":
                            facs.append(f)
                    if not ok:
                        continue
                    r = r_memo[(0,) + tt]
                    coef = " * ".join(facs) if facs else None
                    if expr is None:
                        expr = r if coef is None else f"{coef} * {r}"
                    else:
                        expr = f"{expr} + {r}" if coef is None else f"fma_t({coef}, {r}, {expr})"
                if expr is not None:
                    w(f"  g[{3 * si + d}] = fma_t(dw[{iab}], {expr}, g[{3 * si + d}]);")
    w("}")
    return "\n".join(out)


# (the FP64 code of the larger ones spills registers heavily)
GEN_D_CLASSES = [(0, 0, 2, 0), (0, 0, 2, 1), (1, 0, 2, 0), (2, 0, 0, 0), (2, 0, 1, 0)]


def main():
    pcls = [(0, 0), (1, 0), (1, 1)]
    parts = ["// GENERATED by gen_grad.py -- do not edit by hand.", "#pragma once", ""]
    for (la, lb) in pcls:
        for (lc, ld) in pcls:
            code, _ = gen_class(la, lb, lc, ld)
            parts.append(code)
            parts.append("")
    # (bra class, ket class) combinations with a d pair and few components per
    # quartet; the larger ones use the warp-per-quartet kernels of gradd.cu
    for c in GEN_D_CLASSES:
        code, _ = gen_class(*c)
        parts.append(code)
        parts.append("")
    for (la, lb) in pcls + [(2, 0), (2, 1), (2, 2)]:
        parts.append(gen_vne(la, lb))
        parts.append("")
    Path(__file__).with_name("grad_gen.cuh").write_text("\n".join(parts))


if __name__ == "__main__":
    main()
