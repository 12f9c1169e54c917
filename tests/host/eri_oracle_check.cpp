// Host check of the generated ERI code (csrc/eri_gen.cuh) against the oracle:
// reads one shell quartet per line from stdin - class name, the four centres,
// exponents and contraction coefficients of one primitive per shell - and
// prints the components of (ab|cd) from eri_ketprim_<class> (one bra and one
// ket primitive pair), which tests/test_generated_code_host.py compares with
// the oracle's contracted ERIs of the same one-primitive functions (d
// components in the order xx, xy, xz, yy, yz, zz, one coefficient per shell).
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>
#define __device__
#define __forceinline__ inline
#define __restrict__
enum { BRA_P = 0, BRA_INVP, BRA_PX, BRA_PY, BRA_PZ, BRA_PAX, BRA_PAY, BRA_PAZ, BRA_PBX, BRA_PBY, BRA_PBZ, BRA_K, BRA_AEXP };
#define BRA_SB 16
template <typename T> struct BraPrim { T p, invp, Px, Py, Pz, PAx, PAy, PAz, PBx, PBy, PBz, K, a; };
inline void load_bra_prim(const double* r, BraPrim<double>& b) {
  b.p = r[0]; b.invp = r[1]; b.Px = r[2]; b.Py = r[3]; b.Pz = r[4]; b.PAx = r[5]; b.PAy = r[6]; b.PAz = r[7];
  b.PBx = r[8]; b.PBy = r[9]; b.PBz = r[10]; b.K = r[11]; b.a = r[12];
}
template <typename T> T rsqrt_t(T x) { return 1 / std::sqrt(x); }
template <typename T> T fma_t(T a, T b, T c) { return std::fma(a, b, c); }
// F_m(t) = exp(-t) sum_k (2t)^k / ((2m+1)(2m+3)...(2m+2k+1)), long double
template <typename T, int L> void boys_eval(T t, const T*, T* F) {
  for (int m = 0; m <= L; ++m) {
    long double term = 1.0L / (2 * m + 1), s = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0L * t / (2 * m + 2 * k + 1);
      s += term;
      if (term < 1e-22L * s) break;
    }
    F[m] = (T)(std::exp(-(long double)t) * s);
  }
}
struct Gam { const double* v; double get(int i) const { return v[i]; } };
struct TkA { double* v; double get(int i) const { return v[i]; } void set(int i, double x) { v[i] = x; } };
struct Acc { double v[1296] = {}; double& operator[](int i) { return v[i]; } double get(int i) const { return v[i]; } };
#include "eri_gen.cuh"

static const double SQ2PI54 = std::sqrt(2.0) * std::pow(M_PI, 1.25);
// primitive-pair fields as the device layout holds them, K' = sqrt(2 pi^(5/2)) c_a c_b exp(-mu AB^2) / p
static void pair(const double* A, const double* B, double a, double b, double ca, double cb, double* r) {
  const double p = a + b;
  double P[3], ab2 = 0;
  for (int x = 0; x < 3; ++x) { P[x] = (a * A[x] + b * B[x]) / p; ab2 += (A[x] - B[x]) * (A[x] - B[x]); }
  r[0] = p; r[1] = 1 / p;
  for (int x = 0; x < 3; ++x) { r[2 + x] = P[x]; r[5 + x] = P[x] - A[x]; r[8 + x] = P[x] - B[x]; }
  r[11] = SQ2PI54 * ca * cb * std::exp(-a * b / p * ab2) / p;
  r[12] = a;
}

#define RUN(cls, NOUT)                                                                                        \
  if (name == #cls) {                                                                                         \
    Acc acc;                                                                                                  \
    eri_ketprim_##cls<double, Acc>(sb, 1, BRA_SB, kt[0], kt[1], kt[2], kt[3], kt[4], kt[5], kt[6], kt[7], kt[8], \
                                   kt[9], kt[10], kt[11], nullptr, acc);                                      \
    for (int i = 0; i < NOUT; ++i) std::printf("%.17e%c", acc.v[i], i + 1 < NOUT ? ' ' : '\n');              \
    continue;                                                                                                 \
  }

int main() {
  char buf[16];
  while (std::scanf("%15s", buf) == 1) {
    const std::string name(buf);
    double X[4][3], e[4], c[4];
    for (int k = 0; k < 4; ++k)
      if (std::scanf("%lf %lf %lf", &X[k][0], &X[k][1], &X[k][2]) != 3) return 1;
    for (int k = 0; k < 4; ++k)
      if (std::scanf("%lf", &e[k]) != 1) return 1;
    for (int k = 0; k < 4; ++k)
      if (std::scanf("%lf", &c[k]) != 1) return 1;
    double sb[BRA_SB], kt[BRA_SB];
    pair(X[0], X[1], e[0], e[1], c[0], c[1], sb);
    pair(X[2], X[3], e[2], e[3], c[2], c[3], kt);
    RUN(ssss, 1) RUN(psss, 3) RUN(psps, 9) RUN(sspp, 9) RUN(pspp, 27) RUN(pppp, 81)
    RUN(dsss, 6) RUN(dsps, 18) RUN(dspp, 54) RUN(dsds, 36) RUN(dpss, 18) RUN(dpps, 54) RUN(ddss, 36)
    return 2;
  }
  return 0;
}
