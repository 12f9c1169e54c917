// Host check of the generated integral code (csrc/eri_gen.cuh, csrc/grad_gen.cuh):
// compiled for the CPU with stand-ins for the device helpers (a long-double
// series for the Boys function), it compares the bra-centre derivatives of
// grad_ket_<class> + grad_ketprim_<class> with central differences (h = 1e-4
// bohr) of sum_abcd Gamma_abcd (ab|cd) from eri_ketprim_<class> (or, where
// that class is generated only as (cd|ab), from it with bra and ket
// exchanged), for random centres, exponents and Gamma; prints the largest error
// relative to the largest derivative for each of the 14 generated classes.  Run by tests/test_generated_code_host.py.
#include <cmath>
#include <cstdio>
#include <random>
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
#include "grad_gen.cuh"

static const double SQ2PI54 = std::sqrt(2.0) * std::pow(M_PI, 1.25);
static void pair(const double* A, const double* B, double a, double b, double* r) {
  const double p = a + b;
  double P[3], ab2 = 0;
  for (int x = 0; x < 3; ++x) { P[x] = (a * A[x] + b * B[x]) / p; ab2 += (A[x] - B[x]) * (A[x] - B[x]); }
  r[0] = p; r[1] = 1 / p;
  for (int x = 0; x < 3; ++x) { r[2 + x] = P[x]; r[5 + x] = P[x] - A[x]; r[8 + x] = P[x] - B[x]; }
  r[11] = SQ2PI54 * std::exp(-a * b / p * ab2) / p;
  r[12] = a;
}
std::mt19937_64 rng(11);
static double U(double lo, double hi) { return std::uniform_real_distribution<double>(lo, hi)(rng); }

// E(A, B) = sum Gamma_abcd (ab|cd) from the ERI class ecls: in the gradient's
// orientation (SW = 0) or, for a gradient class whose ERI code exists only as
// (cd|ab), from that class with bra and ket exchanged (SW = 1)
#define ENERGY(ecls, NOUT, NAB, SW)                                                                              \
  [&](const double* A_, const double* B_) {                                                                      \
    double s1[BRA_SB], s2[BRA_SB];                                                                               \
    pair(A_, B_, ea, eb, s1);                                                                                    \
    pair(C, D, ec, ed, s2);                                                                                      \
    const double* sb = SW ? s2 : s1;                                                                             \
    const double* kt = SW ? s1 : s2;                                                                             \
    Acc acc;                                                                                                     \
    eri_ketprim_##ecls<double, Acc>(sb, 1, BRA_SB, kt[0], kt[1], kt[2], kt[3], kt[4], kt[5], kt[6], kt[7], kt[8], \
                                    kt[9], kt[10], kt[11], nullptr, acc);                                        \
    const int NCD = NOUT / NAB;                                                                                  \
    double e = 0;                                                                                                \
    for (int iab = 0; iab < NAB; ++iab)                                                                          \
      for (int icd = 0; icd < NCD; ++icd)                                                                        \
        e += gam[iab * NCD + icd] * acc.v[SW ? icd * NAB + iab : iab * NCD + icd];                               \
    return e;                                                                                                    \
  }

#define CHECK(cls, ecls, NOUT, NAB, SW)                                                                          \
  {                                                                                                              \
    double worst = 0;                                                                                            \
    for (int rep = 0; rep < 6; ++rep) {                                                                          \
      double A[3], B[3], C[3], D[3];                                                                             \
      for (int x = 0; x < 3; ++x) { A[x] = U(-1, 1); B[x] = U(-1, 1); C[x] = U(-1, 1); D[x] = U(-1, 1); }       \
      const double ea = U(0.3, 2), eb = U(0.3, 2), ec = U(0.3, 2), ed = U(0.3, 2);                               \
      std::vector<double> gam(NOUT);                                                                             \
      for (auto& g : gam) g = U(-1, 1);                                                                          \
      auto E = ENERGY(ecls, NOUT, NAB, SW);                                                                      \
      double sb[BRA_SB], kt[BRA_SB];                                                                             \
      pair(A, B, ea, eb, sb);                                                                                    \
      pair(C, D, ec, ed, kt);                                                                                    \
      std::vector<double> tkv(2000);                                                                             \
      TkA tk{tkv.data()};                                                                                        \
      Gam G{gam.data()};                                                                                         \
      grad_ket_##cls<double, Gam, TkA>(kt[1], kt[5], kt[6], kt[7], kt[8], kt[9], kt[10], G, tk);                 \
      double g[6] = {0, 0, 0, 0, 0, 0};                                                                          \
      grad_ketprim_##cls<double, TkA>(sb, 1, BRA_SB, kt[0], kt[2], kt[3], kt[4], kt[11], nullptr, tk, g);        \
      const double h = 1e-4;                                                                                     \
      double scale = 1e-12;                                                                                      \
      for (int i = 0; i < 6; ++i) scale = std::fmax(scale, std::fabs(g[i]));                                     \
      for (int side = 0; side < 2; ++side)                                                                       \
        for (int x = 0; x < 3; ++x) {                                                                            \
          double Ap[3] = {A[0], A[1], A[2]}, Am[3] = {A[0], A[1], A[2]};                                         \
          double Bp[3] = {B[0], B[1], B[2]}, Bm[3] = {B[0], B[1], B[2]};                                         \
          if (side == 0) { Ap[x] += h; Am[x] -= h; } else { Bp[x] += h; Bm[x] -= h; }                            \
          const double fd = (E(Ap, Bp) - E(Am, Bm)) / (2 * h);                                                   \
          worst = std::fmax(worst, std::fabs(fd - g[3 * side + x]) / scale);                                     \
        }                                                                                                        \
    }                                                                                                            \
    std::printf("%s %.3e\n", #cls, worst);                                                                       \
  }

int main() {
  CHECK(ssss, ssss, 1, 1, 0) CHECK(psss, psss, 3, 3, 0) CHECK(psps, psps, 9, 3, 0) CHECK(sspp, sspp, 9, 1, 0)
  CHECK(pspp, pspp, 27, 3, 0) CHECK(pppp, pppp, 81, 9, 0) CHECK(dsss, dsss, 6, 6, 0) CHECK(dsps, dsps, 18, 6, 0)
  // classes whose ERI code is generated in the other orientation only
  CHECK(ssps, psss, 3, 1, 1) CHECK(ppss, sspp, 9, 9, 1) CHECK(ppps, pspp, 27, 9, 1) CHECK(ssds, dsss, 6, 1, 1)
  CHECK(ssdp, dpss, 18, 1, 1) CHECK(psds, dsps, 18, 3, 1)
  return 0;
}
