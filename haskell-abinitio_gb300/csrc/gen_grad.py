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
gen_eri.py.  T depends on the ket primitive only, so it is formed once per
ket primitive (``grad_ket_<class>``, into the caller's storage) and the bra
loop (``grad_ketprim_<class>``) reads it block by block; the last line is
summed axis by axis with partial sums shared by the six components
(``contract_factored``).  The generated file is ``grad_gen.cuh``; run
``python gen_grad.py`` after editing.
"""
from pathlib import Path

from gen_eri import CART, LNAME, e_axis_code, r_code


def lincomb(terms):
    """Expression for sum_k c_k v_k over (c_k, v_k) pairs; c_k 'ONE' is a plain add."""
    expr = None
    for c, v in terms:
        if c == "ONE":
            expr = v if expr is None else f"{expr} + {v}"
        else:
            expr = f"{c} * {v}" if expr is None else f"fma_t({c}, {v}, {expr})"
    return expr


def contract_factored(w, a, b, bmaps, dfac, unames, ind):
    """The six bra-centre components of one bra component pair ab,

        g_S,d += sum_tuv F^S,d_x(t) F^S,d_y(u) F^S,d_z(v) U(tuv),

    with F the Hermite coefficient E^(a_x b_x)_t of each axis except the
    derivative axis d, where it is the derivative factor of side S, summed
    axis by axis (z, then y, then x) so that the partial sums over the
    undifferentiated axes are shared by the components:

        Z0(t,u)  = sum_v E_z(v) U(tuv)           (d = x and d = y)
        Y0(t)    = sum_u E_y(u) Z0(t,u)          g_S,x = sum_t D^S_x(t) Y0(t)
        g_S,y    = sum_t E_x(t) sum_u D^S_y(u) Z0(t,u)
        g_S,z    = sum_t E_x(t) sum_u E_y(u) sum_v D^S_z(v) U(tuv)
    """
    nx, ny, nz = (a[x] + b[x] for x in range(3))

    def E(x, t):
        return bmaps[x].get((a[x], b[x], t))

    def D(side, x, t):
        return dfac(side, x, a[x], b[x], t)

    cnt = [0]

    def emit(expr, terms):
        """A name for the combination: the value itself for one unit term."""
        if expr is None:
            return None
        if len(terms) == 1 and terms[0][0] == "ONE":
            return terms[0][1]
        nm = f"s{cnt[0]}"
        cnt[0] += 1
        w(f"{ind}const T {nm} = {expr};")
        return nm

    def comb(pairs):
        terms = [(c, v) for c, v in pairs if c is not None and v is not None]
        return emit(lincomb(terms), terms)

    z0 = {}
    for t in range(nx + 2):
        for u in range(ny + 2):
            if t == nx + 1 and u == ny + 1:
                continue
            z0[(t, u)] = comb((E(2, v), unames.get((t, u, v))) for v in range(nz + 1))
    y0 = {t: comb((E(1, u), z0.get((t, u))) for u in range(ny + 1)) for t in range(nx + 2)}
    for si, side in enumerate("AB"):
        outs = []
        # d = x
        outs.append(lincomb([(D(side, 0, t), y0[t]) for t in range(nx + 2)
                             if D(side, 0, t) is not None and y0[t] is not None]))
        # d = y
        yy = {t: comb((D(side, 1, u), z0.get((t, u))) for u in range(ny + 2)) for t in range(nx + 1)}
        outs.append(lincomb([(E(0, t), yy[t]) for t in range(nx + 1) if E(0, t) is not None and yy[t] is not None]))
        # d = z
        yz = {}
        for t in range(nx + 1):
            zz = {u: comb((D(side, 2, v), unames.get((t, u, v))) for v in range(nz + 2)) for u in range(ny + 1)}
            yz[t] = comb((E(1, u), zz[u]) for u in range(ny + 1))
        outs.append(lincomb([(E(0, t), yz[t]) for t in range(nx + 1) if E(0, t) is not None and yz[t] is not None]))
        for d, expr in enumerate(outs):
            if expr is not None:
                w(f"{ind}g[{3 * si + d}] += {expr};")


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
    nku = len(ket_union)
    w(f"// ---- gradient class ({cls[0]}{cls[1]}|{cls[2]}{cls[3]}): bra-centre derivatives, L + 1 = {L}")
    w(f"// ket side of one ket primitive pair: T_ab(tau) for ab x {nku} Hermite indices tau")
    w("template <typename T, typename G, typename TK>")
    w(f"__device__ __forceinline__ void grad_ket_{cls}(const T invq,")
    w("    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz, const G& gam, TK& tk) {")
    w("  const T ONE = T(1);")
    w("  (void)ONE; (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;")
    w("  const T hq = T(0.5) * invq;")
    w("  (void)hq;")
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
    # T_ab(tau) = sum_cd Gamma_abcd ekp_cd(tau)
    for (ia, ib) in bra:
        iab = ia * len(cb) + ib
        for k, tau in enumerate(ket_union):
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
            assert expr is not None
            w(f"  tk.set({iab * nku + k}, {expr});")
    w("}")
    w(f"// bra loop of one ket primitive pair, with its T_ab(tau) from grad_ket_{cls}")
    w("template <typename T, typename TK>")
    w(f"__device__ __forceinline__ void grad_ketprim_{cls}(const T* __restrict__ sb, int nbra, int bstep,")
    w("    const T q, const T Qx, const T Qy, const T Qz, const T Kcd, const T* __restrict__ boys,")
    w("    const TK& tk, T* g) {")
    w("  const T ONE = T(1);")
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

    # every derivative factor at loop scope (shared by the ab blocks)
    for (a, b, ds, _) in bra.values():
        for side in "AB":
            for d in range(3):
                for tt in ds[(side, d)]:
                    dfac(side, d, a[d], b[d], tt[d])

    for (ia, ib), (a, b, ds, uset) in bra.items():
        iab = ia * len(cb) + ib
        w("    {")
        tnames = {}
        for k, tau in enumerate(ket_union):
            nm = f"T_{tau[0]}{tau[1]}{tau[2]}"
            w(f"      const T {nm} = tk.get({iab * nku + k});")
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
        contract_factored(w, a, b, bmaps, dfac, unames, "      ")
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


def render():
    """The text of grad_gen.cuh."""
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
    return "\n".join(parts)


def main():
    Path(__file__).with_name("grad_gen.cuh").write_text(render())


if __name__ == "__main__":
    main()
