// CPU FP64 oracle for the RHF hot path.  TEST INFRASTRUCTURE ONLY: it is
// loaded by tests/, by __graft_entry__.smoke() as the checker, and by
// bench.py's CPU-baseline / reference arm.  The product library (libgbhf)
// never links or calls it.
//
// It restates the numerics of felipeZ/Haskell-abinitio (paths relative to the
// reference checkout):
//   Boys function     Science/QuantumChemistry/NumericalTools/Boys.hs:54-118,
//                     NumericalTools/TableBoys.hs:45-69
//   1-e integrals     Integrals/IntegralsEvaluation.hs:169-280, 385-414
//   ERIs              Integrals/IntegralsEvaluation.hs:289-522
//   flat layouts      NumericalTools/LinearAlgebra.hs:240-316
//   Fock from ERIs    HartreeFock/HartreeFock.hs:213-260
// Two numerics presets:
//   ref_compat = 1: Boys values from the reference's 0.1-spaced grid with its
//     6-term floor-point Taylor expansion, grid nodes from 256-point
//     Gauss-Legendre quadrature of Kummer's integral (Boys.hs:106-118 selects
//     nIntegrate256 because 0.1 > 0.1 is false), per-primitive-quartet
//     screening with twoTermsERI at 1e-8, S_ii forced to 1.0.
//   ref_compat = 0: exact Boys function (series / asymptotic + recursion), no
//     primitive screening, true overlap diagonal.
// The direct Fock build (orc_fock_direct) is shell based with contracted
// Schwarz screening and exists so that large systems can be checked and the
// CPU baseline can be timed.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <array>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.141592653589793;

// ------------------------------------------------------------------ Boys ----

// Exact Boys function F_m(x) = int_0^1 t^{2m} exp(-x t^2) dt.
// Small/moderate x: power series F_m(x) = e^{-x} sum_k (2x)^k / ((2m+1)(2m+3)..(2m+2k+1))
// evaluated in long double; large x: F_0 from erf and upward recursion.
double boys_exact_ld(int m, double xd) {
  long double x = xd;
  if (xd < 0) return NAN;
  if (xd > 50.0 && m < 40) {
    long double f = 0.5L * sqrtl((long double)kPi / x) * erfl(sqrtl(x));
    long double ex = expl(-x);
    for (int k = 0; k < m; ++k) f = ((2 * k + 1) * f - ex) / (2 * x);
    return (double)f;
  }
  long double term = 1.0L / (2 * m + 1), sum = term;
  for (int k = 1; k < 2000; ++k) {
    term *= 2 * x / (2 * m + 2 * k + 1);
    sum += term;
    if (term < sum * 1e-21L) break;
  }
  return (double)(expl(-x) * sum);
}

// Fast double-precision F_0..F_mmax (used in the shell-based direct build):
// series for F_mmax then downward recursion; asymptotic + upward for x > 35.
void boys_exact_vec(int mmax, double x, double* f) {
  if (x > 35.0) {
    double ex = std::exp(-x);
    f[0] = 0.5 * std::sqrt(kPi / x) * std::erf(std::sqrt(x));
    for (int k = 0; k < mmax; ++k) f[k + 1] = ((2 * k + 1) * f[k] - ex) / (2 * x);
    return;
  }
  double term = 1.0 / (2 * mmax + 1), sum = term;
  for (int k = 1; k < 400; ++k) {
    term *= 2 * x / (2 * mmax + 2 * k + 1);
    sum += term;
    if (term < sum * 1e-17) break;
  }
  double ex = std::exp(-x);
  f[mmax] = ex * sum;
  for (int k = mmax; k > 0; --k) f[k - 1] = (2 * x * f[k] + ex) / (2 * k - 1);
}

// Gauss-Legendre nodes/weights on [-1,1], n points; returns the n/2 positive
// nodes in ascending order (the layout of PointsWeights.hs points256).
void gauss_legendre_pos(int n, std::vector<double>& xs, std::vector<double>& ws) {
  int half = n / 2;
  xs.assign(half, 0.0);
  ws.assign(half, 0.0);
  for (int i = 0; i < half; ++i) {
    // i-th root counted from x = 1 downwards
    long double z = cosl((long double)kPi * (i + 0.75L) / (n + 0.5L));
    long double pp = 0;
    for (int it = 0; it < 100; ++it) {
      long double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        long double p3 = p2;
        p2 = p1;
        p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      long double z1 = z;
      z = z1 - p1 / pp;
      if (fabsl(z - z1) < 1e-30L) break;
    }
    {
      long double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        long double p3 = p2;
        p2 = p1;
        p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
    }
    xs[half - 1 - i] = (double)z;
    ws[half - 1 - i] = (double)(2.0L / ((1 - z * z) * pp * pp));
  }
}

struct Quad256 {
  std::vector<double> x, w;
  Quad256() { gauss_legendre_pos(256, x, w); }
};
const Quad256& quad256() {
  static Quad256 q;
  return q;
}

// Haskell Int arithmetic (64-bit, wrapping) for fac/facOdd (Boys.hs:89-100).
double fac_odd_hs(long i) {
  auto fac = [](long n) -> int64_t {
    uint64_t p = 1;
    for (long k = 1; k <= n; ++k) p *= (uint64_t)k;
    return (int64_t)p;
  };
  if (i < 2) return 1.0;  // compare i 2 == LT (even i never reaches here)
  long k = (1 + i) / 2;
  return (double)fac(2 * k) / (std::pow(2.0, (double)k) * (double)fac(k));
}

// asymptBoysF (Boys.hs:85-87)
double asympt_boys_ref(double m, double x) {
  double fn = fac_odd_hs((long)std::floor(2 * m - 1));
  return (fn / std::pow(2.0, m + 1)) * std::sqrt(kPi / std::pow(x, 2 * m + 1));
}

// boysF (Boys.hs:54-66) with kummer (Boys.hs:106-118) -> nIntegrate256.
double boys_ref(double n, double x) {
  if (n == 0) {
    if (x > 50) return asympt_boys_ref(0, x);
    if (x > 0.0e-5) return 0.5 * std::sqrt(kPi / x) * std::erf(std::sqrt(x));
    return 1.0;
  }
  const double a = n + 0.5, b = n + 1.5, z = -x;
  const double gamma_factor = std::tgamma(b) / (std::tgamma(a) * std::tgamma(b - a));
  const double e = std::exp(1.0);
  auto fun = [&](double t) {
    return (std::pow(e, z * t) * std::pow(1 - t, b - a - 1)) * std::pow(t, a - 1);
  };
  const Quad256& q = quad256();
  const double lo = 0, hi = 1;
  double acc = 0;
  for (size_t i = 0; i < q.x.size(); ++i) {
    auto g = [&](double xx) { return fun(0.5 * ((hi - lo) * xx + hi + lo)); };
    acc += q.w[i] * (g(q.x[i]) + g(-q.x[i]));
  }
  double integral = 0.5 * (hi - lo) * acc;
  double k = gamma_factor * integral;
  return k / (2 * n + 1);
}

constexpr int kGridM = 15, kGridX = 1001;

// calcBoys (TableBoys.hs:65-69)
inline double calc_boys(const double* grid, int m, double xk) {
  if (xk > 100) return asympt_boys_ref(m, xk);
  long i = std::lround(xk / 0.1);
  return grid[m * kGridX + i];
}

// boysTaylor (TableBoys.hs:45-51)
double boys_taylor(const double* grid, int m, double x) {
  const double delta = 0.1;
  double xk = std::floor(x / delta) * delta;
  double dx = x - xk;
  double dx2 = dx * dx, dx3 = dx2 * dx, dx4 = dx2 * dx2, dx5 = dx4 * dx;
  return calc_boys(grid, m, xk) - calc_boys(grid, m + 1, xk) * dx +
         0.5 * calc_boys(grid, m + 2, xk) * dx2 - (1.0 / 6) * calc_boys(grid, m + 3, xk) * dx3 +
         (1.0 / 24) * calc_boys(grid, m + 4, xk) * dx4 -
         (1.0 / 120) * calc_boys(grid, m + 5, xk) * dx5;
}

// ----------------------------------------------------------------- basis ----

struct Fn {
  int atom;
  int l[3];
  int np, off;
};

struct Shell {
  int atom, L, np;
  int ncomp;
  std::vector<int> fidx;                  // basis-function index per component
  std::vector<std::array<int, 3>> lxyz;   // per component
  std::vector<double> expo;               // np
  std::vector<double> coef;               // ncomp * np (per-component coefficients)
};

struct Basis {
  int natoms = 0;
  std::vector<double> xyz, Z;
  std::vector<Fn> fns;
  std::vector<double> coef, expo;
  std::vector<Shell> shells;
  const double* grid = nullptr;  // reference Boys grid (ref_compat), 15*1001
  int nf() const { return (int)fns.size(); }
  const double* R(int atom) const { return &xyz[3 * atom]; }
};

int ncart(int L) { return (L + 1) * (L + 2) / 2; }

bool same_prims(const Basis& b, const Fn& f, const Fn& g) {
  if (f.np != g.np) return false;
  for (int k = 0; k < f.np; ++k)
    if (b.expo[f.off + k] != b.expo[g.off + k]) return false;
  return true;
}

void build_shells(Basis& b) {
  b.shells.clear();
  int n = b.nf();
  int i = 0;
  while (i < n) {
    const Fn& f = b.fns[i];
    int L = f.l[0] + f.l[1] + f.l[2];
    int nc = ncart(L);
    Shell s;
    s.atom = f.atom;
    s.L = L;
    s.np = f.np;
    s.ncomp = nc;
    s.expo.assign(b.expo.begin() + f.off, b.expo.begin() + f.off + f.np);
    int j = i;
    while (j < n && j < i + nc) {
      const Fn& g = b.fns[j];
      if (g.atom != f.atom || g.l[0] + g.l[1] + g.l[2] != L || !same_prims(b, f, g)) break;
      s.fidx.push_back(j);
      s.lxyz.push_back({g.l[0], g.l[1], g.l[2]});
      for (int k = 0; k < g.np; ++k) s.coef.push_back(b.coef[g.off + k]);
      ++j;
    }
    s.ncomp = (int)s.fidx.size();
    b.shells.push_back(std::move(s));
    i = j;
  }
}

// ------------------------------------------------------------ Hermite E ----

// E[i][j][t] per axis, i<=la, j<=lb, t<=i+j (recursiveHermCoeff,
// IntegralsEvaluation.hs:457-477).  Storage: E[(i*(lb+1)+j)*(la+lb+1)+t].
struct Eaxis {
  int la, lb, T;
  double v[9 * 9 * 9];
  double operator()(int i, int j, int t) const {
    if (i < 0 || j < 0 || t < 0 || t > i + j) return 0.0;
    return v[(i * (lb + 1) + j) * T + t];
  }
};

void hermite_axis(Eaxis& E, int la, int lb, double p, double xpa, double xpb, double e0) {
  E.la = la;
  E.lb = lb;
  E.T = la + lb + 1;
  for (int i = 0; i <= la; ++i)
    for (int j = 0; j <= lb; ++j)
      for (int t = 0; t <= i + j; ++t) {
        double val;
        if (i == 0 && j == 0 && t == 0) {
          val = e0;
        } else if (t == 0 && i >= 1) {
          val = xpa * E(i - 1, j, 0) + E(i - 1, j, 1);
        } else if (t == 0) {
          val = xpb * E(i, j - 1, 0) + E(i, j - 1, 1);
        } else {
          val = (1.0 / (2 * p * t)) * (i * E(i - 1, j, t - 1) + j * E(i, j - 1, t - 1));
        }
        E.v[(i * (lb + 1) + j) * E.T + t] = val;
      }
}

// ------------------------------------------------------------ Hermite R ----

// R^0_{tuv}(alpha, X, Y, Z) for t+u+v <= L (calcHermM, IntegralsEvaluation.hs:430-449).
struct Rtab {
  int L;
  std::vector<double> r;  // (L+1)^3 at n = 0
  double operator()(int t, int u, int v) const { return r[(t * (L + 1) + u) * (L + 1) + v]; }
};

void hermite_r(Rtab& R, int L, double alpha, double X, double Y, double Z, const double* F) {
  // F[n] = F_n(T), n = 0..L.  Work array Rn[n][t][u][v].
  int d = L + 1;
  std::vector<double> w((size_t)d * d * d * d, 0.0);
  auto at = [&](int n, int t, int u, int v) -> double& { return w[((n * d + t) * d + u) * d + v]; };
  double m2a = -2 * alpha, pw = 1;
  for (int n = 0; n <= L; ++n) {
    at(n, 0, 0, 0) = pw * F[n];
    pw *= m2a;
  }
  for (int n = L - 1; n >= 0; --n) {
    int top = L - n;
    for (int s = 1; s <= top; ++s)
      for (int t = 0; t <= s; ++t)
        for (int u = 0; u <= s - t; ++u) {
          int v = s - t - u;
          double val;
          if (t >= 1) {
            val = (t >= 2 ? (t - 1) * at(n + 1, t - 2, u, v) : 0.0) + X * at(n + 1, t - 1, u, v);
          } else if (u >= 1) {
            val = (u >= 2 ? (u - 1) * at(n + 1, t, u - 2, v) : 0.0) + Y * at(n + 1, t, u - 1, v);
          } else {
            val = (v >= 2 ? (v - 1) * at(n + 1, t, u, v - 2) : 0.0) + Z * at(n + 1, t, u, v - 1);
          }
          at(n, t, u, v) = val;
        }
  }
  R.L = L;
  R.r.assign((size_t)d * d * d, 0.0);
  for (int t = 0; t <= L; ++t)
    for (int u = 0; u + t <= L; ++u)
      for (int v = 0; v + u + t <= L; ++v) R.r[(t * d + u) * d + v] = at(0, t, u, v);
}

void boys_values(const Basis& b, bool ref, int L, double T, double* F) {
  if (ref) {
    for (int n = 0; n <= L; ++n) F[n] = boys_taylor(b.grid, n, T);
  } else {
    boys_exact_vec(L, T, F);
  }
}

// ----------------------------------------------------- one-electron terms ----

// obaraSaika (IntegralsEvaluation.hs:209-221)
double obara_saika(double gamma, double s00, double pax, double pbx, int m, int n) {
  if (m < 0 || n < 0) return 0;
  if (m == 0 && n == 0) return s00;
  double c = 1.0 / (2.0 * gamma);
  double m1 = m - 1, n1 = n - 1;
  if (m == 0) return pbx * obara_saika(gamma, s00, pax, pbx, 0, n - 1) + c * n1 * obara_saika(gamma, s00, pax, pbx, 0, n - 2);
  if (n == 0) return pax * obara_saika(gamma, s00, pax, pbx, m - 1, 0) + c * m1 * obara_saika(gamma, s00, pax, pbx, m - 2, 0);
  return pax * obara_saika(gamma, s00, pax, pbx, m - 1, n) +
         c * (m1 * obara_saika(gamma, s00, pax, pbx, m - 2, n) + n * obara_saika(gamma, s00, pax, pbx, m - 1, n - 1));
}

struct PrimPair {
  double p, mu, P[3], PA[3], PB[3], AB[3];
};

PrimPair make_pair(const double* A, const double* B, double a, double b) {
  PrimPair q;
  q.p = a + b;
  q.mu = a * b / q.p;
  for (int x = 0; x < 3; ++x) {
    q.P[x] = (a * A[x] + b * B[x]) / (a + b);
    q.PA[x] = q.P[x] - A[x];
    q.PB[x] = q.P[x] - B[x];
    q.AB[x] = A[x] - B[x];
  }
  return q;
}

double overlap_fn(const Basis& b, int i, int j, bool ref) {
  const Fn &f = b.fns[i], &g = b.fns[j];
  const double *A = b.R(f.atom), *B = b.R(g.atom);
  if (ref) {
    // sijContracted short-circuit (IntegralsEvaluation.hs:183-184): identical CGF on one centre
    bool same = f.l[0] == g.l[0] && f.l[1] == g.l[1] && f.l[2] == g.l[2] && f.np == g.np &&
                A[0] == B[0] && A[1] == B[1] && A[2] == B[2];
    for (int k = 0; same && k < f.np; ++k)
      same = b.coef[f.off + k] == b.coef[g.off + k] && b.expo[f.off + k] == b.expo[g.off + k];
    if (same) return 1.0;
  }
  double s = 0;
  for (int p1 = 0; p1 < f.np; ++p1)
    for (int p2 = 0; p2 < g.np; ++p2) {
      double c1 = b.coef[f.off + p1], e1 = b.expo[f.off + p1];
      double c2 = b.coef[g.off + p2], e2 = b.expo[g.off + p2];
      PrimPair q = make_pair(A, B, e1, e2);
      double cte = std::sqrt(kPi / q.p), prod = 1;
      for (int x = 0; x < 3; ++x) {
        double s00 = std::exp(-q.mu * q.AB[x] * q.AB[x]) * cte;
        prod *= obara_saika(q.p, s00, q.PA[x], q.PB[x], f.l[x], g.l[x]);
      }
      s += (c1 * c2) * prod;
    }
  return s;
}

// tab (IntegralsEvaluation.hs:263-280)
double kinetic_fn(const Basis& b, int i, int j) {
  const Fn &f = b.fns[i], &g = b.fns[j];
  const double *A = b.R(f.atom), *B = b.R(g.atom);
  double s = 0;
  for (int p1 = 0; p1 < f.np; ++p1)
    for (int p2 = 0; p2 < g.np; ++p2) {
      double c1 = b.coef[f.off + p1], e1 = b.expo[f.off + p1];
      double c2 = b.coef[g.off + p2], e2 = b.expo[g.off + p2];
      PrimPair q = make_pair(A, B, e1, e2);
      double cte = std::sqrt(kPi / q.p);
      double sx[3], tx[3];
      for (int x = 0; x < 3; ++x) {
        double s00 = std::exp(-q.mu * q.AB[x] * q.AB[x]) * cte;
        int l1 = f.l[x], l2 = g.l[x];
        sx[x] = obara_saika(q.p, s00, q.PA[x], q.PB[x], l1, l2);
        tx[x] = -2.0 * e2 * e2 * obara_saika(q.p, s00, q.PA[x], q.PB[x], l1, l2 + 2) +
                e2 * (2 * l2 + 1) * obara_saika(q.p, s00, q.PA[x], q.PB[x], l1, l2) -
                0.5 * l2 * (l2 - 1) * obara_saika(q.p, s00, q.PA[x], q.PB[x], l1, l2 - 2);
      }
      s += c1 * c2 * (tx[0] * sx[1] * sx[2] + sx[0] * tx[1] * sx[2] + sx[0] * sx[1] * tx[2]);
    }
  return s;
}

// vijContracted / vijHermite / mcMurchie (IntegralsEvaluation.hs:385-414)
double nuclear_fn(const Basis& b, int i, int j, const double* C, bool ref) {
  const Fn &f = b.fns[i], &g = b.fns[j];
  const double *A = b.R(f.atom), *B = b.R(g.atom);
  int L = f.l[0] + f.l[1] + f.l[2] + g.l[0] + g.l[1] + g.l[2];
  double s = 0;
  double F[32];
  Eaxis E[3];
  Rtab R;
  for (int p1 = 0; p1 < f.np; ++p1)
    for (int p2 = 0; p2 < g.np; ++p2) {
      double c1 = b.coef[f.off + p1], e1 = b.expo[f.off + p1];
      double c2 = b.coef[g.off + p2], e2 = b.expo[g.off + p2];
      PrimPair q = make_pair(A, B, e1, e2);
      for (int x = 0; x < 3; ++x)
        hermite_axis(E[x], f.l[x], g.l[x], q.p, q.PA[x], q.PB[x], std::exp(-q.mu * q.AB[x] * q.AB[x]));
      double PC[3] = {q.P[0] - C[0], q.P[1] - C[1], q.P[2] - C[2]};
      double T = q.p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
      boys_values(b, ref, L, T, F);
      hermite_r(R, L, q.p, PC[0], PC[1], PC[2], F);
      double sum = 0;
      for (int t = 0; t <= f.l[0] + g.l[0]; ++t)
        for (int u = 0; u <= f.l[1] + g.l[1]; ++u)
          for (int v = 0; v <= f.l[2] + g.l[2]; ++v)
            sum += E[0](f.l[0], g.l[0], t) * E[1](f.l[1], g.l[1], u) * E[2](f.l[2], g.l[2], v) * R(t, u, v);
      s += c1 * c2 * 2.0 * (kPi / q.p) * sum;
    }
  return s;
}

// -------------------------------------------------------- ERIs (per fn) ----

struct GPrim {
  const double* R;
  int l[3];
  double c, e;
};

// twoTermsERI (IntegralsEvaluation.hs:319-337)
double two_terms_eri(const GPrim& ga, const GPrim& gb) {
  PrimPair q = make_pair(ga.R, gb.R, ga.e, gb.e);
  Eaxis E[3];
  for (int x = 0; x < 3; ++x)
    hermite_axis(E[x], ga.l[x], gb.l[x], q.p, q.PA[x], q.PB[x], std::exp(-q.mu * q.AB[x] * q.AB[x]));
  double sum_c = 0, sum_s = 0;
  for (int t = 0; t <= ga.l[0] + gb.l[0]; ++t)
    for (int u = 0; u <= ga.l[1] + gb.l[1]; ++u)
      for (int v = 0; v <= ga.l[2] + gb.l[2]; ++v) {
        double e = E[0](ga.l[0], gb.l[0], t) * E[1](ga.l[1], gb.l[1], u) * E[2](ga.l[2], gb.l[2], v);
        sum_c += e;
        sum_s += ((t + u + v) % 2 ? -1.0 : 1.0) * e;
      }
  double x = kPi / (2 * q.p);
  double x2 = x * x;
  double cte = 2 * ((ga.c * ga.c) * (gb.c * gb.c)) * std::sqrt(x2 * x2 * x);
  return cte * (sum_c * sum_s);
}

// twoElectronHermite (IntegralsEvaluation.hs:340-376) for one primitive quartet.
double two_electron_hermite(const Basis& b, bool ref, const GPrim* g) {
  PrimPair ab = make_pair(g[0].R, g[1].R, g[0].e, g[1].e);
  PrimPair cd = make_pair(g[2].R, g[3].R, g[2].e, g[3].e);
  Eaxis E1[3], E2[3];
  for (int x = 0; x < 3; ++x) {
    hermite_axis(E1[x], g[0].l[x], g[1].l[x], ab.p, ab.PA[x], ab.PB[x], std::exp(-ab.mu * ab.AB[x] * ab.AB[x]));
    hermite_axis(E2[x], g[2].l[x], g[3].l[x], cd.p, cd.PA[x], cd.PB[x], std::exp(-cd.mu * cd.AB[x] * cd.AB[x]));
  }
  double p = ab.p, q = cd.p, alpha = p * q / (p + q);
  double PQ[3] = {ab.P[0] - cd.P[0], ab.P[1] - cd.P[1], ab.P[2] - cd.P[2]};
  int lab[3], lcd[3], L = 0;
  for (int x = 0; x < 3; ++x) {
    lab[x] = g[0].l[x] + g[1].l[x];
    lcd[x] = g[2].l[x] + g[3].l[x];
    L += lab[x] + lcd[x];
  }
  double F[40];
  boys_values(b, ref, L, alpha * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]), F);
  Rtab R;
  hermite_r(R, L, alpha, PQ[0], PQ[1], PQ[2], F);
  double total = 0;
  for (int t = 0; t <= lab[0]; ++t)
    for (int u = 0; u <= lab[1]; ++u)
      for (int v = 0; v <= lab[2]; ++v) {
        double e1 = E1[0](g[0].l[0], g[1].l[0], t) * E1[1](g[0].l[1], g[1].l[1], u) * E1[2](g[0].l[2], g[1].l[2], v);
        double inner = 0;
        for (int tau = 0; tau <= lcd[0]; ++tau)
          for (int nu = 0; nu <= lcd[1]; ++nu)
            for (int phi = 0; phi <= lcd[2]; ++phi) {
              double e2 = E2[0](g[2].l[0], g[3].l[0], tau) * E2[1](g[2].l[1], g[3].l[1], nu) *
                          E2[2](g[2].l[2], g[3].l[2], phi);
              double sg = ((tau + nu + phi) % 2) ? -1.0 : 1.0;
              inner += sg * e2 * R(t + tau, u + nu, v + phi);
            }
        total += e1 * inner;
      }
  double cte = (g[0].c * g[1].c * g[2].c * g[3].c) * ((2.0 * std::pow(kPi, 2.5)) * (1.0 / ((p * q) * std::sqrt(p + q))));
  return cte * total;
}

// contracted4Centers (IntegralsEvaluation.hs:294-315)
double eri_fn(const Basis& b, bool ref, int i, int j, int k, int l) {
  const Fn* f[4] = {&b.fns[i], &b.fns[j], &b.fns[k], &b.fns[l]};
  GPrim g[4];
  for (int a = 0; a < 4; ++a) {
    g[a].R = b.R(f[a]->atom);
    for (int x = 0; x < 3; ++x) g[a].l[x] = f[a]->l[x];
  }
  double sum = 0;
  for (int p1 = 0; p1 < f[0]->np; ++p1) {
    g[0].c = b.coef[f[0]->off + p1];
    g[0].e = b.expo[f[0]->off + p1];
    for (int p2 = 0; p2 < f[1]->np; ++p2) {
      g[1].c = b.coef[f[1]->off + p2];
      g[1].e = b.expo[f[1]->off + p2];
      double qab = ref ? std::sqrt(two_terms_eri(g[0], g[1])) : 0.0;
      for (int p3 = 0; p3 < f[2]->np; ++p3) {
        g[2].c = b.coef[f[2]->off + p3];
        g[2].e = b.expo[f[2]->off + p3];
        for (int p4 = 0; p4 < f[3]->np; ++p4) {
          g[3].c = b.coef[f[3]->off + p4];
          g[3].e = b.expo[f[3]->off + p4];
          if (ref) {
            double qcd = std::sqrt(two_terms_eri(g[2], g[3]));
            double val = qab * qcd;
            if (val < 1e-8) continue;  // guard (schwarz gauss): keeps NaN
          }
          sum += two_electron_hermite(b, ref, g);
        }
      }
    }
  }
  return sum;
}

// ---------------------------------------------------------- flat indices ----

inline long tri(long n) { return n * (n + 1) / 2; }
// indexDIM2toFlat (LinearAlgebra.hs:250-253) for 0 <= x,y < dim
inline long flat2(long dim, long x, long y) {
  if (x > y) std::swap(x, y);
  return x * dim - tri(x - 1) + (y - x);
}

// Offset of the canonical key block (i,j) in calcIntegrals order
// (HartreeFock.hs:166-181): keys i<=j, k>=i, l>=k with (i,j) <= (k,l).
struct CanonIndex {
  long n;
  std::vector<long> off;  // n*n, valid for i<=j
  explicit CanonIndex(long n_) : n(n_), off(n_ * n_, 0) {
    long acc = 0;
    for (long i = 0; i < n; ++i)
      for (long j = i; j < n; ++j) {
        off[i * n + j] = acc;
        acc += (n - j) + tri(n - i - 1);
      }
  }
  long total() const { return tri(tri(n)); }
  // sorted key (i<=j, k<=l, (i,j) <= (k,l))
  long operator()(long i, long j, long k, long l) const {
    long idx = off[i * n + j];
    if (k == i) return idx + (l - j);
    idx += n - j;
    // sum_{k'=i+1}^{k-1} (n - k')
    long m = k - i - 1;
    idx += m * n - (m * (i + 1) + tri(m - 1));
    return idx + (l - k);
  }
  static void sort_key(long& i, long& j, long& k, long& l) {
    if (i > j) std::swap(i, j);
    if (k > l) std::swap(k, l);
    if (i > k || (i == k && j > l)) {
      std::swap(i, k);
      std::swap(j, l);
    }
  }
};

// -------------------------------------------------- shell-level direct J/K ----

struct ShellPair {
  int A, B;
  double Q;  // sqrt(max_comp (ab|ab))
};

// All component integrals of a shell quartet, layout [a][b][c][d].
void eri_shell_quartet(const Basis& bs, const Shell& A, const Shell& B, const Shell& C, const Shell& D,
                       double* out) {
  const int na = A.ncomp, nb = B.ncomp, nc = C.ncomp, nd = D.ncomp;
  std::fill(out, out + na * nb * nc * nd, 0.0);
  const double *RA = bs.R(A.atom), *RB = bs.R(B.atom), *RC = bs.R(C.atom), *RD = bs.R(D.atom);
  const int L = A.L + B.L + C.L + D.L;
  double F[40];
  Eaxis E1[3], E2[3];
  Rtab R;
  std::vector<double> W;  // [c][d][t][u][v] ket-contracted Hermite intermediate
  const int Lab = A.L + B.L, Lcd = C.L + D.L, d1 = Lab + 1;
  W.assign((size_t)nc * nd * d1 * d1 * d1, 0.0);
  for (int pa = 0; pa < A.np; ++pa)
    for (int pb = 0; pb < B.np; ++pb) {
      PrimPair ab = make_pair(RA, RB, A.expo[pa], B.expo[pb]);
      for (int x = 0; x < 3; ++x)
        hermite_axis(E1[x], A.L, B.L, ab.p, ab.PA[x], ab.PB[x], std::exp(-ab.mu * ab.AB[x] * ab.AB[x]));
      for (int pc = 0; pc < C.np; ++pc)
        for (int pd = 0; pd < D.np; ++pd) {
          PrimPair cd = make_pair(RC, RD, C.expo[pc], D.expo[pd]);
          for (int x = 0; x < 3; ++x)
            hermite_axis(E2[x], C.L, D.L, cd.p, cd.PA[x], cd.PB[x], std::exp(-cd.mu * cd.AB[x] * cd.AB[x]));
          double p = ab.p, q = cd.p, alpha = p * q / (p + q);
          double PQ[3] = {ab.P[0] - cd.P[0], ab.P[1] - cd.P[1], ab.P[2] - cd.P[2]};
          boys_exact_vec(L, alpha * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]), F);
          hermite_r(R, L, alpha, PQ[0], PQ[1], PQ[2], F);
          double pref = 2.0 * std::pow(kPi, 2.5) / (p * q * std::sqrt(p + q));
          // ket contraction into W, then bra contraction into out (per component)
          for (int ic = 0; ic < nc; ++ic)
            for (int id = 0; id < nd; ++id) {
              const auto &lc = C.lxyz[ic], &ld = D.lxyz[id];
              double cc = C.coef[ic * C.np + pc] * D.coef[id * D.np + pd];
              double* w = &W[((size_t)ic * nd + id) * d1 * d1 * d1];
              for (int t = 0; t <= Lab; ++t)
                for (int u = 0; u + t <= Lab; ++u)
                  for (int v = 0; v + u + t <= Lab; ++v) {
                    double inner = 0;
                    for (int tau = 0; tau <= lc[0] + ld[0]; ++tau) {
                      double ex = E2[0](lc[0], ld[0], tau);
                      if (ex == 0) continue;
                      for (int nu = 0; nu <= lc[1] + ld[1]; ++nu) {
                        double ey = E2[1](lc[1], ld[1], nu);
                        for (int phi = 0; phi <= lc[2] + ld[2]; ++phi) {
                          double ez = E2[2](lc[2], ld[2], phi);
                          double sg = ((tau + nu + phi) & 1) ? -1.0 : 1.0;
                          inner += sg * ex * ey * ez * R(t + tau, u + nu, v + phi);
                        }
                      }
                    }
                    w[(t * d1 + u) * d1 + v] = cc * inner;
                  }
            }
          for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
              const auto &la = A.lxyz[ia], &lb = B.lxyz[ib];
              double cab = pref * A.coef[ia * A.np + pa] * B.coef[ib * B.np + pb];
              for (int icd = 0; icd < nc * nd; ++icd) {
                const double* w = &W[(size_t)icd * d1 * d1 * d1];
                double s = 0;
                for (int t = 0; t <= la[0] + lb[0]; ++t) {
                  double ex = E1[0](la[0], lb[0], t);
                  for (int u = 0; u <= la[1] + lb[1]; ++u) {
                    double ey = E1[1](la[1], lb[1], u);
                    for (int v = 0; v <= la[2] + lb[2]; ++v)
                      s += ex * ey * E1[2](la[2], lb[2], v) * w[(t * d1 + u) * d1 + v];
                  }
                }
                out[(ia * nb + ib) * nc * nd + icd] += cab * s;
              }
            }
        }
    }
  (void)Lcd;
}

std::vector<ShellPair> make_shell_pairs(const Basis& b) {
  std::vector<ShellPair> out;
  int ns = (int)b.shells.size();
  std::vector<double> buf;
  for (int A = 0; A < ns; ++A)
    for (int B = 0; B <= A; ++B) {
      const Shell &sa = b.shells[A], &sb = b.shells[B];
      int n = sa.ncomp * sb.ncomp;
      buf.assign((size_t)n * n, 0.0);
      eri_shell_quartet(b, sa, sb, sa, sb, buf.data());
      double mx = 0;
      for (int i = 0; i < n; ++i) mx = std::max(mx, std::fabs(buf[(size_t)i * n + i]));
      out.push_back({A, B, std::sqrt(mx)});
    }
  return out;
}

}  // namespace

// =================================================================== C ABI ===
extern "C" {

int orc_version() { return 3; }

double orc_boys_exact(int m, double x) { return boys_exact_ld(m, x); }

void orc_boys_exact_vec(int mmax, double x, double* out) { boys_exact_vec(mmax, x, out); }

void orc_gauss_legendre(int n, double* nodes, double* weights) {
  std::vector<double> x, w;
  gauss_legendre_pos(n, x, w);
  std::memcpy(nodes, x.data(), sizeof(double) * x.size());
  std::memcpy(weights, w.data(), sizeof(double) * w.size());
}

double orc_boys_ref(double m, double x) { return boys_ref(m, x); }

double orc_asympt_boys_ref(double m, double x) { return asympt_boys_ref(m, x); }

// generateGridBoys 0.1 (TableBoys.hs:58-63): grid[m*1001 + i] = boysF m (0.1*i)
void orc_boys_ref_grid(double* grid) {
#pragma omp parallel for schedule(dynamic)
  for (int m = 0; m < kGridM; ++m)
    for (int i = 0; i < kGridX; ++i) grid[m * kGridX + i] = boys_ref((double)m, 0.1 * i);
}

double orc_boys_taylor(const double* grid, int m, double x) { return boys_taylor(grid, m, x); }

void* orc_basis_create(int natoms, const double* xyz, const double* Z, int ncgf, const int* cgf_atom,
                       const int* cgf_lxyz, const int* cgf_nprim, const double* coef, const double* expo,
                       const double* grid) {
  Basis* b = new Basis;
  b->natoms = natoms;
  b->xyz.assign(xyz, xyz + 3 * natoms);
  b->Z.assign(Z, Z + natoms);
  int off = 0;
  for (int i = 0; i < ncgf; ++i) {
    Fn f;
    f.atom = cgf_atom[i];
    for (int x = 0; x < 3; ++x) f.l[x] = cgf_lxyz[3 * i + x];
    f.np = cgf_nprim[i];
    f.off = off;
    off += f.np;
    b->fns.push_back(f);
  }
  b->coef.assign(coef, coef + off);
  b->expo.assign(expo, expo + off);
  b->grid = grid;  // caller keeps it alive (may be null for exact mode)
  build_shells(*b);
  return b;
}

void orc_basis_destroy(void* h) { delete (Basis*)h; }

int orc_nshells(void* h) { return (int)((Basis*)h)->shells.size(); }

void orc_shell_info(void* h, int* atom, int* L, int* ncomp, int* nprim, int* first_fn) {
  Basis* b = (Basis*)h;
  for (size_t s = 0; s < b->shells.size(); ++s) {
    atom[s] = b->shells[s].atom;
    L[s] = b->shells[s].L;
    ncomp[s] = b->shells[s].ncomp;
    nprim[s] = b->shells[s].np;
    first_fn[s] = b->shells[s].fidx[0];
  }
}

// mtxOverlap (IntegralsEvaluation.hs:169-177), flat upper triangle
void orc_overlap(void* h, int ref_compat, double* S) {
  Basis* b = (Basis*)h;
  int n = b->nf();
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) S[flat2(n, i, j)] = overlap_fn(*b, i, j, ref_compat != 0);
}

void orc_kinetic(void* h, double* T) {
  Basis* b = (Basis*)h;
  int n = b->nf();
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) T[flat2(n, i, j)] = kinetic_fn(*b, i, j);
}

// hcore (IntegralsEvaluation.hs:227-240): T - sum_C Z_C V_C
void orc_hcore(void* h, int ref_compat, double* H) {
  Basis* b = (Basis*)h;
  int n = b->nf();
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      double v = 0;
      for (int c = 0; c < b->natoms; ++c) v += (-b->Z[c]) * nuclear_fn(*b, i, j, b->R(c), ref_compat != 0);
      H[flat2(n, i, j)] = kinetic_fn(*b, i, j) + v;
    }
}

// calcIntegrals (HartreeFock.hs:166-181): all canonical ERIs in key order.
long orc_eri_canonical_len(int n) { return (long)tri(tri(n)); }

void orc_eri_canonical(void* h, int ref_compat, double* eri) {
  Basis* b = (Basis*)h;
  long n = b->nf();
  CanonIndex ci(n);
#pragma omp parallel for schedule(dynamic)
  for (long i = 0; i < n; ++i)
    for (long j = i; j < n; ++j)
      for (long k = i; k < n; ++k)
        for (long l = k; l < n; ++l) {
          if (k == i && l < j) continue;
          eri[ci(i, j, k, l)] = eri_fn(*b, ref_compat != 0, (int)i, (int)j, (int)k, (int)l);
        }
}

// Index of a (sorted) key in the canonical array.
long orc_canonical_index(int n, int i, int j, int k, int l) {
  CanonIndex ci(n);
  long a = i, bb = j, c = k, d = l;
  CanonIndex::sort_key(a, bb, c, d);
  return ci(a, bb, c, d);
}

// One contracted ERI (function indices), either numerics preset.
double orc_eri(void* h, int ref_compat, int i, int j, int k, int l) {
  return eri_fn(*(Basis*)h, ref_compat != 0, i, j, k, l);
}

// fock/calcGmatrix (HartreeFock.hs:213-241): F_ab = H_ab + sum_kl D_lk [(ab|kl) - 1/2 (al|kb)]
void orc_fock_canonical(int n, const double* H, const double* D, const double* eri, double* F) {
  CanonIndex ci(n);
  auto E = [&](long i, long j, long k, long l) {
    CanonIndex::sort_key(i, j, k, l);
    return eri[ci(i, j, k, l)];
  };
#pragma omp parallel for schedule(dynamic)
  for (long a = 0; a < n; ++a)
    for (long b = a; b < n; ++b) {
      double g = 0;
      for (long l = 0; l < n; ++l)
        for (long k = 0; k < n; ++k) g += D[flat2(n, l, k)] * (E(a, b, k, l) - 0.5 * E(a, l, k, b));
      F[flat2(n, a, b)] = H[flat2(n, a, b)] + g;
    }
}

// Direct shell-based J/K Fock build (exact numerics).  Skips shell quartets
// with Q_AB*Q_CD < schwarz and, with density_screen, those whose bound times
// the largest |D| over the six density blocks the quartet touches (AB, CD, AC,
// AD, BC, BD) is below schwarz.  stats[0] = computed shell quartets,
// stats[1] = computed primitive quartets, stats[2] = skipped shell quartets.
void orc_fock_direct(void* h, const double* H, const double* D, double schwarz, int density_screen, double* F,
                     long long* stats) {
  Basis* b = (Basis*)h;
  const int n = b->nf();
  std::vector<ShellPair> pairs = make_shell_pairs(*b);
  const long np = (long)pairs.size();
  std::vector<double> Dsq((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Dsq[(size_t)i * n + j] = D[flat2(n, i, j)];
  std::vector<double> G((size_t)n * n, 0.0);
  long long nq = 0, npq = 0, nskip = 0;
#pragma omp parallel reduction(+ : nq, npq, nskip)
  {
    std::vector<double> Gl((size_t)n * n, 0.0), buf;
#pragma omp for schedule(dynamic, 1)
    for (long pab = 0; pab < np; ++pab) {
      const ShellPair& P = pairs[pab];
      const Shell &A = b->shells[P.A], &B = b->shells[P.B];
      for (long pcd = 0; pcd <= pab; ++pcd) {
        const ShellPair& Q = pairs[pcd];
        if (P.Q * Q.Q < schwarz) {
          ++nskip;
          continue;
        }
        const Shell &C = b->shells[Q.A], &Dd = b->shells[Q.B];
        const int na = A.ncomp, nb = B.ncomp, nc = C.ncomp, nd = Dd.ncomp;
        if (density_screen) {
          double dm = 0;
          auto blk = [&](const Shell& X, const Shell& Y) {
            for (int x = 0; x < X.ncomp; ++x)
              for (int y = 0; y < Y.ncomp; ++y) dm = std::max(dm, std::fabs(Dsq[(size_t)X.fidx[x] * n + Y.fidx[y]]));
          };
          blk(A, B);
          blk(C, Dd);
          blk(A, C);
          blk(A, Dd);
          blk(B, C);
          blk(B, Dd);
          if (P.Q * Q.Q * dm < schwarz) {
            ++nskip;
            continue;
          }
        }
        buf.resize((size_t)na * nb * nc * nd);
        eri_shell_quartet(*b, A, B, C, Dd, buf.data());
        ++nq;
        npq += (long long)A.np * B.np * C.np * Dd.np;
        double s = 1.0;
        if (P.A == P.B) s *= 0.5;
        if (Q.A == Q.B) s *= 0.5;
        if (pab == pcd) s *= 0.5;
        for (int ia = 0; ia < na; ++ia)
          for (int ib = 0; ib < nb; ++ib)
            for (int ic = 0; ic < nc; ++ic)
              for (int id = 0; id < nd; ++id) {
                double w = s * buf[((ia * nb + ib) * nc + ic) * nd + id];
                int a = A.fidx[ia], bb = B.fidx[ib], c = C.fidx[ic], d = Dd.fidx[id];
                Gl[(size_t)a * n + bb] += 2 * w * Dsq[(size_t)c * n + d];
                Gl[(size_t)c * n + d] += 2 * w * Dsq[(size_t)a * n + bb];
                Gl[(size_t)a * n + c] -= 0.5 * w * Dsq[(size_t)bb * n + d];
                Gl[(size_t)bb * n + c] -= 0.5 * w * Dsq[(size_t)a * n + d];
                Gl[(size_t)a * n + d] -= 0.5 * w * Dsq[(size_t)bb * n + c];
                Gl[(size_t)bb * n + d] -= 0.5 * w * Dsq[(size_t)a * n + c];
              }
      }
    }
#pragma omp critical
    for (size_t i = 0; i < G.size(); ++i) G[i] += Gl[i];
  }
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) F[flat2(n, i, j)] = H[flat2(n, i, j)] + G[(size_t)i * n + j] + G[(size_t)j * n + i];
  if (stats) {
    stats[0] = nq;
    stats[1] = npq;
    stats[2] = nskip;
  }
}

// Shell-pair Schwarz bounds, in the order A >= B (A outer).
void orc_shell_pair_bounds(void* h, double* Q) {
  std::vector<ShellPair> p = make_shell_pairs(*(Basis*)h);
  for (size_t i = 0; i < p.size(); ++i) Q[i] = p[i].Q;
}

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
