// Generic (runtime angular momentum) McMurchie-Davidson helpers, FP64.
// Used for the one-electron matrices, the canonical ERI array, Schwarz
// bounds and reference-numerics work; the direct J/K build uses the
// generated per-class code instead.
#pragma once
#include "gbhf_common.cuh"

namespace gbhf {

constexpr int MD_LMAX = 4;          // default total angular momentum (s,p quartets; d one-electron)
constexpr int MD_D = MD_LMAX + 1;

struct DevFn {   // one contracted Gaussian
  int atom, l[3], np, off;
};

__device__ __forceinline__ DevFn load_fn(const int* __restrict__ fn, int i) {
  DevFn f;
  f.atom = fn[6 * i];
  f.l[0] = fn[6 * i + 1];
  f.l[1] = fn[6 * i + 2];
  f.l[2] = fn[6 * i + 3];
  f.np = fn[6 * i + 4];
  f.off = fn[6 * i + 5];
  return f;
}

// Hermite E^{ij}_t for one axis, i,j <= 2 (recursiveHermCoeff,
// Integrals/IntegralsEvaluation.hs:457-477), E^{00}_0 = e0.
struct EAx {
  double v[3][3][5];
  __device__ double get(int i, int j, int t) const {
    if (i < 0 || j < 0 || t < 0 || t > i + j) return 0.0;
    return v[i][j][t];
  }
};

__device__ inline void e_axis(EAx& E, int la, int lb, double p, double xpa, double xpb, double e0) {
  for (int i = 0; i <= la; ++i)
    for (int j = 0; j <= lb; ++j)
      for (int t = 0; t <= i + j; ++t) {
        double val;
        if (i == 0 && j == 0 && t == 0) {
          val = e0;
        } else if (t == 0 && i >= 1) {
          val = xpa * E.get(i - 1, j, 0) + E.get(i - 1, j, 1);
        } else if (t == 0) {
          val = xpb * E.get(i, j - 1, 0) + E.get(i, j - 1, 1);
        } else {
          val = (1.0 / (2 * p * t)) * (i * E.get(i - 1, j, t - 1) + j * E.get(i, j - 1, t - 1));
        }
        E.v[i][j][t] = val;
      }
}

// Reference Boys: asymptBoysF (Boys.hs:85-87) with Haskell's wrapping Int
// factorials, and boysTaylor over the 0.1 grid (TableBoys.hs:45-69).
__device__ inline double fac_odd_hs(long i) {
  if (i < 2) return 1.0;
  long k = (1 + i) / 2;
  unsigned long long a = 1, b = 1;
  for (long q = 1; q <= 2 * k; ++q) a *= (unsigned long long)q;
  for (long q = 1; q <= k; ++q) b *= (unsigned long long)q;
  return (double)(long long)a / (pow(2.0, (double)k) * (double)(long long)b);
}

__device__ inline double asympt_boys_ref(double m, double x) {
  double fn = fac_odd_hs((long)floor(2 * m - 1));
  return (fn / pow(2.0, m + 1)) * sqrt(GBHF_PI / pow(x, 2 * m + 1));
}

__device__ inline double calc_boys_ref(const double* __restrict__ grid, int m, long i, double xk) {
  if (xk > 100) return asympt_boys_ref((double)m, xk);
  return grid[m * 1001 + i];
}

__device__ inline double boys_taylor_ref(const double* __restrict__ grid, int m, double x) {
  const double delta = 0.1;
  double fi = floor(x / delta);
  double xk = fi * delta;
  long i = (long)fi;
  double dx = x - xk;
  double dx2 = dx * dx, dx3 = dx2 * dx, dx4 = dx2 * dx2, dx5 = dx4 * dx;
  return calc_boys_ref(grid, m, i, xk) - calc_boys_ref(grid, m + 1, i, xk) * dx +
         0.5 * calc_boys_ref(grid, m + 2, i, xk) * dx2 - (1.0 / 6) * calc_boys_ref(grid, m + 3, i, xk) * dx3 +
         (1.0 / 24) * calc_boys_ref(grid, m + 4, i, xk) * dx4 -
         (1.0 / 120) * calc_boys_ref(grid, m + 5, i, xk) * dx5;
}

// F_0..F_L(T), L <= MD_LMAX (+ a few for derivative work): reference grid or exact table.
__device__ inline void boys_generic(bool ref, const double* __restrict__ grid, const double* __restrict__ tab,
                                    int L, double T, double* F) {
  if (ref) {
    for (int n = 0; n <= L; ++n) F[n] = boys_taylor_ref(grid, n, T);
    return;
  }
  if (T < BOYS64_TMAX) {
    const int j = (int)(T * (1.0 / BOYS64_H) + 0.5);
    const double dx = j * BOYS64_H - T;
    double y[BOYS64_NTERM];
    y[0] = 1;
    for (int k = 1; k < BOYS64_NTERM; ++k) y[k] = y[k - 1] * dx * (1.0 / k);
    const double* row = tab + j * BOYS_NCOL;
    for (int m = 0; m <= L; ++m) {
      double s = 0;
      for (int k = BOYS64_NTERM - 1; k >= 0; --k) s = fma(y[k], row[m + k], s);
      F[m] = s;
    }
  } else {
    const double r = rsqrt(T);
    F[0] = 0.886226925452758 * r;
    const double h = 0.5 * r * r;
    for (int m = 1; m <= L; ++m) F[m] = F[m - 1] * (2 * m - 1) * h;
  }
}

// R^0_{tuv}(alpha, X, Y, Z), t+u+v <= L, from F_n (calcHermM,
// Integrals/IntegralsEvaluation.hs:430-449).  Two-level scheme: level n is
// built from level n+1.  Output cube R[(t*D+u)*D+v], D = LM + 1.
template <int LM>
__device__ inline void hermite_r(int L, double alpha, double X, double Y, double Z, const double* F, double* R) {
  constexpr int D = LM + 1;
  double nxt[D * D * D];
  double pw[LM + 1];
  pw[0] = 1.0;
  for (int n = 1; n <= L; ++n) pw[n] = pw[n - 1] * (-2.0 * alpha);
  nxt[0] = pw[L] * F[L];
  for (int n = L - 1; n >= 0; --n) {
    const int top = L - n;
    // level n from level n+1 (held in nxt for t+u+v <= top-1)
    for (int s = top; s >= 1; --s)
      for (int t = 0; t <= s; ++t)
        for (int u = 0; u <= s - t; ++u) {
          const int v = s - t - u;
          double val;
          if (t >= 1) {
            val = (t >= 2 ? (t - 1) * nxt[((t - 2) * D + u) * D + v] : 0.0) + X * nxt[((t - 1) * D + u) * D + v];
          } else if (u >= 1) {
            val = (u >= 2 ? (u - 1) * nxt[(t * D + u - 2) * D + v] : 0.0) + Y * nxt[(t * D + u - 1) * D + v];
          } else {
            val = (v >= 2 ? (v - 1) * nxt[(t * D + u) * D + v - 2] : 0.0) + Z * nxt[(t * D + u) * D + v - 1];
          }
          R[(t * D + u) * D + v] = val;
        }
    R[0] = pw[n] * F[n];
    for (int s = 0; s <= top; ++s)
      for (int t = 0; t <= s; ++t)
        for (int u = 0; u <= s - t; ++u) {
          const int v = s - t - u;
          nxt[(t * D + u) * D + v] = R[(t * D + u) * D + v];
        }
  }
  if (L == 0) R[0] = nxt[0];
}

// twoTermsERI (Integrals/IntegralsEvaluation.hs:319-337) for a primitive pair.
__device__ inline double two_terms_eri(const double* A, const int* la, double ca, double ea, const double* B,
                                       const int* lb, double cb, double eb) {
  double p = ea + eb, mu = ea * eb / p;
  EAx E[3];
  for (int x = 0; x < 3; ++x) {
    double P = (ea * A[x] + eb * B[x]) / p;
    double ab = A[x] - B[x];
    e_axis(E[x], la[x], lb[x], p, P - A[x], P - B[x], exp(-mu * ab * ab));
  }
  double sc = 0, ss = 0;
  for (int t = 0; t <= la[0] + lb[0]; ++t)
    for (int u = 0; u <= la[1] + lb[1]; ++u)
      for (int v = 0; v <= la[2] + lb[2]; ++v) {
        double e = E[0].get(la[0], lb[0], t) * E[1].get(la[1], lb[1], u) * E[2].get(la[2], lb[2], v);
        sc += e;
        ss += ((t + u + v) & 1) ? -e : e;
      }
  double xx = GBHF_PI / (2 * p);
  double x2 = xx * xx;
  double cte = 2 * ((ca * ca) * (cb * cb)) * sqrt(x2 * x2 * xx);
  return cte * (sc * ss);
}

// One contracted ERI (ab|cd) over CGFs (contracted4Centers,
// Integrals/IntegralsEvaluation.hs:294-306); ref enables the per-primitive
// screening of schwarz (:308-315) and reference Boys.
template <int LM = MD_LMAX>
__device__ inline double eri_fn_generic(bool ref, const double* __restrict__ xyz, const int* __restrict__ fn,
                                        const double* __restrict__ coef, const double* __restrict__ expo,
                                        const double* __restrict__ grid, const double* __restrict__ tab, int i,
                                        int j, int k, int l, int r0 = 0, int rstep = 1) {
  // the primitive quartets (p1 p2 | p3 p4) in nested-loop order r, this call
  // summing r = r0, r0 + rstep, ... (r0 = 0, rstep = 1: all of them, in order)
  DevFn f[4] = {load_fn(fn, i), load_fn(fn, j), load_fn(fn, k), load_fn(fn, l)};
  const double* R4[4];
  for (int a = 0; a < 4; ++a) R4[a] = xyz + 3 * f[a].atom;
  int lab[3], lcd[3], L = 0;
  for (int x = 0; x < 3; ++x) {
    lab[x] = f[0].l[x] + f[1].l[x];
    lcd[x] = f[2].l[x] + f[3].l[x];
    L += lab[x] + lcd[x];
  }
  constexpr int D = LM + 1;
  double sum = 0;
  double F[LM + 1];
  double R[D * D * D];
  EAx E1[3], E2[3];
  const int n2 = f[1].np, n3 = f[2].np, n4 = f[3].np, nr = f[0].np * n2 * n3 * n4;
  int last12 = -1;
  double c12 = 0, qab = 0, p = 0, P[3] = {0, 0, 0};
  for (int r = r0; r < nr; r += rstep) {
    const int p4 = r % n4, r3 = r / n4, p3 = r3 % n3, r12 = r3 / n3, p2 = r12 % n2, p1 = r12 / n2;
    if (r12 != last12) {
      last12 = r12;
      const double c1 = coef[f[0].off + p1], e1 = expo[f[0].off + p1];
      const double c2 = coef[f[1].off + p2], e2 = expo[f[1].off + p2];
      c12 = c1 * c2;
      qab = ref ? sqrt(two_terms_eri(R4[0], f[0].l, c1, e1, R4[1], f[1].l, c2, e2)) : 0.0;
      p = e1 + e2;
      const double mu = e1 * e2 / p;
      for (int x = 0; x < 3; ++x) {
        P[x] = (e1 * R4[0][x] + e2 * R4[1][x]) / p;
        double ab = R4[0][x] - R4[1][x];
        e_axis(E1[x], f[0].l[x], f[1].l[x], p, P[x] - R4[0][x], P[x] - R4[1][x], exp(-mu * ab * ab));
      }
    }
    const double c3 = coef[f[2].off + p3], e3 = expo[f[2].off + p3];
    const double c4 = coef[f[3].off + p4], e4 = expo[f[3].off + p4];
    if (ref) {
      double qcd = sqrt(two_terms_eri(R4[2], f[2].l, c3, e3, R4[3], f[3].l, c4, e4));
      if (qab * qcd < 1e-8) continue;   // !(val < 1e-8) keeps NaN, as guard (schwarz gs)
    }
    const double q = e3 + e4, nu = e3 * e4 / q;
    double Q[3], PQ[3];
    for (int x = 0; x < 3; ++x) {
      Q[x] = (e3 * R4[2][x] + e4 * R4[3][x]) / q;
      double cd = R4[2][x] - R4[3][x];
      e_axis(E2[x], f[2].l[x], f[3].l[x], q, Q[x] - R4[2][x], Q[x] - R4[3][x], exp(-nu * cd * cd));
      PQ[x] = P[x] - Q[x];
    }
    const double alpha = p * q / (p + q);
    boys_generic(ref, grid, tab, L, alpha * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]), F);
    hermite_r<LM>(L, alpha, PQ[0], PQ[1], PQ[2], F, R);
    double total = 0;
    for (int t = 0; t <= lab[0]; ++t)
      for (int u = 0; u <= lab[1]; ++u)
        for (int v = 0; v <= lab[2]; ++v) {
          double eb = E1[0].get(f[0].l[0], f[1].l[0], t) * E1[1].get(f[0].l[1], f[1].l[1], u) *
                      E1[2].get(f[0].l[2], f[1].l[2], v);
          double inner = 0;
          for (int tau = 0; tau <= lcd[0]; ++tau)
            for (int nu2 = 0; nu2 <= lcd[1]; ++nu2)
              for (int phi = 0; phi <= lcd[2]; ++phi) {
                double ek = E2[0].get(f[2].l[0], f[3].l[0], tau) * E2[1].get(f[2].l[1], f[3].l[1], nu2) *
                            E2[2].get(f[2].l[2], f[3].l[2], phi);
                double rr = R[((t + tau) * D + (u + nu2)) * D + (v + phi)];
                inner += ((tau + nu2 + phi) & 1) ? -ek * rr : ek * rr;
              }
          total += eb * inner;
        }
    const double cte = (c12 * c3 * c4) * ((2.0 * 17.493418327624862) * (1.0 / ((p * q) * sqrt(p + q))));
    sum += cte * total;
  }
  return sum;
}

}  // namespace gbhf
