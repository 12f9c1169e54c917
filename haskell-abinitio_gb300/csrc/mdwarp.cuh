// Warp-cooperative McMurchie-Davidson evaluation of one contracted shell
// quartet, for the quartet classes that hold a d shell.
//
// Those classes have many Cartesian components ((dd|dd): 1296 integrals per
// quartet) and few primitives (the d shells of the Pople sets have one), so
// one warp evaluates one quartet at a time and its 32 lanes share each stage
// of a primitive quartet through shared memory:
//   R^n_tuv   Hermite Coulomb integrals of every order n <= L - (t+u+v), built
//             level by level in t+u+v from R^n_000 = pref (-2 alpha)^n F_n(T);
//   X[h][cd]  = sum_(tau nu phi) (-1)^(tau+nu+phi) E^cd_(tau nu phi) R^0_(h + (tau nu phi));
//   (ab|cd)  += sum_h E^ab_h X[h][cd].
// These are the sums of twoElectronHermite / mcMurchie2 / calcHermIntegral
// (Integrals/IntegralsEvaluation.hs:340-376, 418-449) with the Hermite
// expansion coefficients of calcHermCoeff (:452-477), restated per warp.
//
// Cartesian components of a shell follow the reference's CGF order
// (BasisSet/FetchBasis.hs:50-59): p = x, y, z; d = xx, xy, xz, yy, yz, zz.
// The components of a d shell carry different primitive normalisations; the
// shell keeps the coefficients of its first component and a constant ratio
// (scale) per component, applied where the contracted integrals are used.
#pragma once
#include "gbhf_common.cuh"

namespace gbhf {

__host__ __device__ constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
// Hermite index of (t, u, v): levels s = t+u+v in order, inside a level by (u+v, v).
__host__ __device__ constexpr int hidx(int t, int u, int v) {
  return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + (u + v) * (u + v + 1) / 2 + v;
}

// Cartesian exponents (lx, ly) of component c of a shell of angular momentum L <= 2;
// lz = L - lx - ly.  Two bits per component: d = xx xy xz yy yz zz.
__device__ __forceinline__ void cart_exps(int L, int c, int& lx, int& ly, int& lz) {
  if (L == 2) {
    lx = (22 >> (2 * c)) & 3;
    ly = (388 >> (2 * c)) & 3;
  } else if (L == 1) {
    lx = c == 0;
    ly = c == 1;
  } else {
    lx = 0;
    ly = 0;
  }
  lz = L - lx - ly;
}

// Sizes and shared-memory layout (elements of T per warp) of one class.
// DERIV = 1: the bra Hermite range and E tables grow by one for the
// bra-centre derivatives of the gradient.
template <int LA, int LB, int LC, int LD, int DERIV>
struct MDCfg {
  static constexpr int LA_ = LA, LB_ = LB, LC_ = LC, LD_ = LD;
  static constexpr int LAe = LA + DERIV, LBe = LB + DERIV;
  static constexpr int LAB = LA + LB + DERIV, LCD = LC + LD, L = LAB + LCD;
  static constexpr int NA = (LA + 1) * (LA + 2) / 2, NB = (LB + 1) * (LB + 2) / 2;
  static constexpr int NC = (LC + 1) * (LC + 2) / 2, ND = (LD + 1) * (LD + 2) / 2;
  static constexpr int NAB = NA * NB, NCD = NC * ND, NOUT = NAB * NCD;
  static constexpr int NR = nherm(L), NHAB = nherm(LAB);
  static constexpr int EBD = LAe + LBe + 1, EKD = LCD + 1;              // t extent of one E table row
  static constexpr int EB = (LAe + 1) * (LBe + 1) * EBD, EK = (LC + 1) * (LD + 1) * EKD;
  static constexpr int SZ_R = (L + 1) * NR;
  static constexpr int OFF_R = 0;
  static constexpr int OFF_X = OFF_R + SZ_R;
  static constexpr int OFF_EB = OFF_X + NHAB * NCD;
  static constexpr int OFF_EK = OFF_EB + 3 * EB;
  static constexpr int OFF_G = OFF_EK + 3 * EK;                        // Gamma (gradient)
  static constexpr int OFF_SB = ((OFF_G + (DERIV ? NOUT : 0)) + 3) & ~3;   // staged bra primitives, 32-byte aligned
  static constexpr int WS = OFF_SB + KMAX_PRIM_PAIRS * BRA_SB;
  static constexpr int NPL = (NOUT + 31) / 32;                           // integrals per lane
  static_assert(SZ_R >= NOUT, "the R area holds the contracted block for the scatter");
};

// E^{ij}_t of one axis for i <= li, j <= lj (row (i, j) of length TD), written
// by one lane: E^{00}_0 = 1 (exp(-mu X_AB^2) sits in the pair prefactor),
// E^{i+1,j}_t = E^{ij}_(t-1)/(2p) + X_PA E^{ij}_t + (t+1) E^{ij}_(t+1), and the
// same in j with X_PB.
template <int LI, int LJ, int TD, typename T>
__device__ __forceinline__ void md_e_axis(T* E, T h2p, T pa, T pb) {
  for (int k = 0; k < (LI + 1) * (LJ + 1) * TD; ++k) E[k] = T(0);
  E[0] = T(1);
  for (int i = 0; i <= LI; ++i)
    for (int j = 0; j <= LJ; ++j) {
      if (i == 0 && j == 0) continue;
      const bool up_i = i > 0;
      const T* src = up_i ? E + ((i - 1) * (LJ + 1) + j) * TD : E + (i * (LJ + 1) + j - 1) * TD;
      const int ts = i + j - 1;   // top t of the source row
      const T x = up_i ? pa : pb;
      T* dst = E + (i * (LJ + 1) + j) * TD;
      for (int t = 0; t <= i + j; ++t) {
        T v = T(0);
        if (t >= 1) v = h2p * src[t - 1];
        if (t <= ts) v = fma_t(x, src[t], v);
        if (t + 1 <= ts) v = fma_t(T(t + 1), src[t + 1], v);
        dst[t] = v;
      }
    }
}

// Primitive data of one side of a quartet.
template <typename T>
struct MDPrim {
  T p, invp, P[3], PA[3], PB[3], K;
};

// The Hermite stages of one primitive quartet, up to X (lane-parallel, ends
// with __syncwarp).  Lanes 0-2 must have written the bra E tables already;
// lanes 3-5 write the ket E tables here.  tuv: (t | u << 8 | v << 16) of every
// Hermite index up to L.
template <class C, typename T>
__device__ __forceinline__ void md_prim_x(T* ws, const int* __restrict__ tuv, const MDPrim<T>& bp,
                                          const MDPrim<T>& kp, const T* __restrict__ boys, int lane) {
  constexpr int L = C::L, NR = C::NR;
  T* R = ws + C::OFF_R;
  T* X = ws + C::OFF_X;
  if (lane >= 3 && lane < 6) {
    const int x = lane - 3;
    md_e_axis<C::LC_, C::LD_, C::EKD>(ws + C::OFF_EK + x * C::EK, T(0.5) * kp.invp, kp.PA[x], kp.PB[x]);
  }
  const T X0 = bp.P[0] - kp.P[0], Y0 = bp.P[1] - kp.P[1], Z0 = bp.P[2] - kp.P[2];
  const T ppq = bp.p + kp.p;
  const T rs = rsqrt_t(ppq);
  const T alpha = bp.p * kp.p * (rs * rs);
  const T Tb = alpha * (X0 * X0 + Y0 * Y0 + Z0 * Z0);
  T F[L + 1];
  boys_eval<T, L>(Tb, boys, F);
  {
    const T m2a = T(-2) * alpha;
    T fac = bp.K * kp.K * rs;
#pragma unroll
    for (int m = 0; m <= L; ++m) {
      if (lane == m) R[m * NR] = fac * F[m];
      fac *= m2a;
    }
  }
  __syncwarp();
  // levels s = 1..L: R^n_tuv for n <= L - s from order n+1 of levels s-1, s-2
#pragma unroll 1
  for (int s = 1; s <= L; ++s) {
    const int nlev = (s + 1) * (s + 2) / 2, base = s * (s + 1) * (s + 2) / 6;
    const int tot = (L - s + 1) * nlev;
    for (int e = lane; e < tot; e += 32) {
      const int n = e / nlev, pos = e - n * nlev;
      const int w = tuv[base + pos];
      const int t = w & 255, u = (w >> 8) & 255, v = w >> 16;
      const T* R1 = R + (n + 1) * NR;
      T val;
      if (t > 0) {
        val = X0 * R1[hidx(t - 1, u, v)];
        if (t > 1) val = fma_t(T(t - 1), R1[hidx(t - 2, u, v)], val);
      } else if (u > 0) {
        val = Y0 * R1[hidx(t, u - 1, v)];
        if (u > 1) val = fma_t(T(u - 1), R1[hidx(t, u - 2, v)], val);
      } else {
        val = Z0 * R1[hidx(t, u, v - 1)];
        if (v > 1) val = fma_t(T(v - 1), R1[hidx(t, u, v - 2)], val);
      }
      R[n * NR + base + pos] = val;
    }
    __syncwarp();
  }
  // ket transformation
  const T* Ekx = ws + C::OFF_EK;
  const T* Eky = Ekx + C::EK;
  const T* Ekz = Eky + C::EK;
  for (int e = lane; e < C::NHAB * C::NCD; e += 32) {
    const int h = e / C::NCD, cd = e - h * C::NCD;
    const int w = tuv[h];
    const int t = w & 255, u = (w >> 8) & 255, v = w >> 16;
    const int ic = cd / C::ND, id = cd - ic * C::ND;
    int cx, cy, cz, dx, dy, dz;
    cart_exps(C::LC_, ic, cx, cy, cz);
    cart_exps(C::LD_, id, dx, dy, dz);
    const T* ex = Ekx + (cx * (C::LD_ + 1) + dx) * C::EKD;
    const T* ey = Eky + (cy * (C::LD_ + 1) + dy) * C::EKD;
    const T* ez = Ekz + (cz * (C::LD_ + 1) + dz) * C::EKD;
    T sum = T(0);
    for (int ta = 0; ta <= cx + dx; ++ta)
      for (int ua = 0; ua <= cy + dy; ++ua) {
        const T exy = ex[ta] * ey[ua];
        for (int va = 0; va <= cz + dz; ++va) {
          const T r = exy * ez[va] * R[hidx(t + ta, u + ua, v + va)];
          sum += ((ta + ua + va) & 1) ? -r : r;
        }
      }
    X[e] = sum;
  }
  __syncwarp();
}

// Bra E tables of one primitive pair (lanes 0-2).
template <class C, typename T>
__device__ __forceinline__ void md_bra_e(T* ws, const MDPrim<T>& bp, int lane) {
  if (lane < 3) md_e_axis<C::LAe, C::LBe, C::EBD>(ws + C::OFF_EB + lane * C::EB, T(0.5) * bp.invp, bp.PA[lane], bp.PB[lane]);
}

// Bra transformation for the J/K integrals: lane-owned entries e = lane + 32 k
// of the NAB x NCD block, acc[k] += sum_h E^ab_h X[h][cd].
template <class C, typename T>
__device__ __forceinline__ void md_bra_acc(const T* ws, T* acc, int lane) {
  const T* X = ws + C::OFF_X;
  const T* Ebx = ws + C::OFF_EB;
  const T* Eby = Ebx + C::EB;
  const T* Ebz = Eby + C::EB;
#pragma unroll
  for (int k = 0; k < C::NPL; ++k) {
    const int e = lane + 32 * k;
    if (e < C::NOUT) {
      const int ab = e / C::NCD, cd = e - ab * C::NCD;
      const int ia = ab / C::NB, ib = ab - ia * C::NB;
      int ax, ay, az, bx, by, bz;
      cart_exps(C::LA_, ia, ax, ay, az);
      cart_exps(C::LB_, ib, bx, by, bz);
      const T* ex = Ebx + (ax * (C::LBe + 1) + bx) * C::EBD;
      const T* ey = Eby + (ay * (C::LBe + 1) + by) * C::EBD;
      const T* ez = Ebz + (az * (C::LBe + 1) + bz) * C::EBD;
      T sum = T(0);
      for (int t = 0; t <= ax + bx; ++t)
        for (int u = 0; u <= ay + by; ++u) {
          const T exy = ex[t] * ey[u];
          for (int v = 0; v <= az + bz; ++v) sum = fma_t(exy * ez[v], X[hidx(t, u, v) * C::NCD + cd], sum);
        }
      acc[k] += sum;
    }
  }
}

// Bra transformation for the gradient: bra-centre derivatives of the
// primitive quartet contracted with Gamma (OFF_G, NAB x NCD), added to
// g[0..5] = d/dA_xyz, d/dB_xyz.  d/dA_x of a Cartesian Gaussian is
// 2 a G(l_x + 1) - l_x G(l_x - 1), so the derivative integrals use the bra E
// tables one order up in i (for A) or j (for B).
template <class C, typename T>
__device__ __forceinline__ void md_bra_grad(const T* ws, const int* __restrict__ tuv, T ea, T eb, T* g, int lane) {
  const T* X = ws + C::OFF_X;
  const T* Gm = ws + C::OFF_G;
  const T* Eb = ws + C::OFF_EB;
  auto E = [&](int x, int i, int j, int t) -> T {
    return (i < 0 || j < 0 || t > i + j) ? T(0) : Eb[x * C::EB + (i * (C::LBe + 1) + j) * C::EBD + t];
  };
  for (int e = lane; e < C::NAB * C::NHAB; e += 32) {
    const int ab = e / C::NHAB, h = e - ab * C::NHAB;
    const int w = tuv[h];
    const int t = w & 255, u = (w >> 8) & 255, v = w >> 16;
    const int ia = ab / C::NB, ib = ab - ia * C::NB;
    int ax, ay, az, bx, by, bz;
    cart_exps(C::LA_, ia, ax, ay, az);
    cart_exps(C::LB_, ib, bx, by, bz);
    const int Tx = ax + bx, Ty = ay + by, Tz = az + bz;
    const bool in0 = t <= Tx && u <= Ty && v <= Tz;
    const bool okx = t <= Tx + 1 && u <= Ty && v <= Tz;
    const bool oky = t <= Tx && u <= Ty + 1 && v <= Tz;
    const bool okz = t <= Tx && u <= Ty && v <= Tz + 1;
    if (!(in0 || okx || oky || okz)) continue;
    T z = T(0);
    const T* xr = X + h * C::NCD;
    const T* gr = Gm + ab * C::NCD;
    for (int cd = 0; cd < C::NCD; ++cd) z = fma_t(gr[cd], xr[cd], z);
    const T ex0 = E(0, ax, bx, t), ey0 = E(1, ay, by, u), ez0 = E(2, az, bz, v);
    const T dax = T(2) * ea * E(0, ax + 1, bx, t) - T(ax) * E(0, ax - 1, bx, t);
    const T day = T(2) * ea * E(1, ay + 1, by, u) - T(ay) * E(1, ay - 1, by, u);
    const T daz = T(2) * ea * E(2, az + 1, bz, v) - T(az) * E(2, az - 1, bz, v);
    const T dbx = T(2) * eb * E(0, ax, bx + 1, t) - T(bx) * E(0, ax, bx - 1, t);
    const T dby = T(2) * eb * E(1, ay, by + 1, u) - T(by) * E(1, ay, by - 1, u);
    const T dbz = T(2) * eb * E(2, az, bz + 1, v) - T(bz) * E(2, az, bz - 1, v);
    const T yz = ey0 * ez0 * z, xz = ex0 * ez0 * z, xy = ex0 * ey0 * z;
    g[0] = fma_t(dax, yz, g[0]);
    g[1] = fma_t(day, xz, g[1]);
    g[2] = fma_t(daz, xy, g[2]);
    g[3] = fma_t(dbx, yz, g[3]);
    g[4] = fma_t(dby, xz, g[4]);
    g[5] = fma_t(dbz, xy, g[5]);
  }
}

// (t | u << 8 | v << 16) of every Hermite index up to L, filled once per block.
__device__ __forceinline__ void md_fill_tuv(int* tuv, int L) {
  const int n = nherm(L);
  for (int h = threadIdx.x; h < n; h += blockDim.x) {
    int s = 0;
    while (nherm(s) <= h) ++s;
    const int pos = h - (s > 0 ? nherm(s - 1) : 0);
    int a = 0;
    while ((a + 1) * (a + 2) / 2 <= pos) ++a;
    const int v = pos - a * (a + 1) / 2, u = a - v, t = s - a;
    tuv[h] = t | (u << 8) | (v << 16);
  }
}

// Primitive pair k of a pair in field-major layout (field f at base[f * npp + idx]).
template <typename T>
__device__ __forceinline__ void md_load_prim(const T* __restrict__ base, long long npp, long long idx, MDPrim<T>& pr) {
  pr.p = base[BRA_P * npp + idx];
  pr.invp = base[BRA_INVP * npp + idx];
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    pr.P[x] = base[(BRA_PX + x) * npp + idx];
    pr.PA[x] = base[(BRA_PAX + x) * npp + idx];
    pr.PB[x] = base[(BRA_PBX + x) * npp + idx];
  }
  pr.K = base[BRA_K * npp + idx];
}

// The same from a staged row (BRA_SB fields of one primitive pair).
template <typename T>
__device__ __forceinline__ void md_row_prim(const T* __restrict__ row, MDPrim<T>& pr) {
  pr.p = row[BRA_P];
  pr.invp = row[BRA_INVP];
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    pr.P[x] = row[BRA_PX + x];
    pr.PA[x] = row[BRA_PAX + x];
    pr.PB[x] = row[BRA_PBX + x];
  }
  pr.K = row[BRA_K];
}

}  // namespace gbhf
