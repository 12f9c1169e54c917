// Shared device-side definitions for libgbhf (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define TWO_PI_2P5 34.98683665524972   // 2 pi^(5/2)
#define GBHF_PI 3.141592653589793

// Boys tables: F_m(T_j) on a uniform grid, row j holds m = 0 .. BOYS_NCOL-1.
#define BOYS_NCOL 16
// FP64: spacing 0.025 up to 60, 6-term Taylor about the nearest node (the
// remainder |dx|^6 / 6! F_(m+6) <= 5e-15 F_m with |dx| <= 0.0125; one FMA per
// Horner evaluation fewer than 7 terms at spacing 0.05, on the FP64 pipe that
// bounds the FP64 ERI kernels).  Beyond TMAX the asymptotic form drops a term
// of relative size exp(-T) T^(m-1/2) / Gamma(m+1/2): below 1e-16 for m <= 9 at
// T = 60.
#define BOYS64_H 0.025
#define BOYS64_TMAX 60.0
#define BOYS64_NROW 2402
#define BOYS64_NTERM 6
// FP32: spacing 0.05 up to 36, 4-term Taylor about the nearest node (remainder
// |dx|^4 / 4! F_(m+4) <= 1.7e-8 F_m with |dx| <= 0.025, below the FP32 rounding
// of the sum; the asymptotic term above is below 4e-8 for m <= 9 at T = 36).
#define BOYS32_H 0.05f
#define BOYS32_TMAX 36.0f
#define BOYS32_NROW 722
#define BOYS32_NTERM 4

// Bra primitive-pair fields (shared-memory staging and global SoA layout).
enum {
  BRA_P = 0, BRA_INVP, BRA_PX, BRA_PY, BRA_PZ, BRA_PAX, BRA_PAY, BRA_PAZ,
  BRA_PBX, BRA_PBY, BRA_PBZ, BRA_K, BRA_AEXP, BRA_NFIELD
};
// Cartesian components of a shell of angular momentum L.
constexpr int ncart_c(int L) { return (L + 1) * (L + 2) / 2; }
// Hermite indices (t, u, v) with t + u + v <= L.
constexpr int nherm_c(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// The J/K kernels stage the first BRA_NJK fields; BRA_AEXP (the exponent of
// the pair's first primitive) is read by the gradient kernels only.
#define BRA_NJK BRA_AEXP
#define KMAX_PRIM_PAIRS 36   // primitive pairs per shell pair (6 x 6)
// A bra primitive pair staged in shared memory: its fields contiguous, padded
// to 16 values so that every row starts on a 16-byte boundary and is read with
// vector loads (7 x 16 bytes for double, 4 x 16 bytes for float).
#define BRA_SB 16

template <typename T>
struct BraPrim {
  T p, invp, Px, Py, Pz, PAx, PAy, PAz, PBx, PBy, PBz, K, a;
};
__device__ __forceinline__ void load_bra_prim(const double* __restrict__ r, BraPrim<double>& b) {
  const double2* v = reinterpret_cast<const double2*>(r);
  const double2 x0 = v[0], x1 = v[1], x2 = v[2], x3 = v[3], x4 = v[4], x5 = v[5], x6 = v[6];
  b.p = x0.x, b.invp = x0.y, b.Px = x1.x, b.Py = x1.y, b.Pz = x2.x, b.PAx = x2.y, b.PAy = x3.x;
  b.PAz = x3.y, b.PBx = x4.x, b.PBy = x4.y, b.PBz = x5.x, b.K = x5.y, b.a = x6.x;
}
__device__ __forceinline__ void load_bra_prim(const float* __restrict__ r, BraPrim<float>& b) {
  const float4* v = reinterpret_cast<const float4*>(r);
  const float4 x0 = v[0], x1 = v[1], x2 = v[2], x3 = v[3];
  b.p = x0.x, b.invp = x0.y, b.Px = x0.z, b.Py = x0.w, b.Pz = x1.x, b.PAx = x1.y, b.PAy = x1.z;
  b.PAz = x1.w, b.PBx = x2.x, b.PBy = x2.y, b.PBz = x2.z, b.K = x2.w, b.a = x3.x;
}

// 1/sqrt(x) in FP64 with few FP64-pipe instructions (that pipe is 1/64 of the
// FP32 rate on this GPU): x is truncated to single precision by moving its
// exponent and top mantissa bits (integer ops), the single-precision estimate
// rsqrtf (relative error ~2^-21 with the truncation) is widened the same way,
// and one second-order Newton (Householder) step y (1 + e/2 + 3e^2/8),
// e = 1 - x y^2, brings it to ~1 ulp (the neglected term is ~(5/16) e^3).
// Valid for positive normal x with 2^-126 < x < 2^127 (every caller passes an
// exponent sum or a Boys argument >= 20).
__device__ __forceinline__ double rsqrt_d(double x) {
  const int hi = __double2hiint(x);
  const float xf = __int_as_float((hi - 0x38000000) << 3);
  const int yb = __float_as_int(rsqrtf(xf));
  const double y = __hiloint2double((yb >> 3) + 0x38000000, yb << 29);
  const double e = fma(-x, y * y, 1.0);
  return fma(y * e, fma(0.375, e, 0.5), y);
}

// float -> double without the conversion instruction (which runs on the FP64
// pipe): the exponent is rebiased and the mantissa shifted with integer ops.
// Zeros and float denormals (|x| < 1.2e-38) give 0; the FP32 kernels never
// produce Inf or NaN from finite data.
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) {
  const int b = __float_as_int(x);
  if ((b & 0x7f800000) == 0) return 0.0;
  const int hi = (b & (int)0x80000000) | ((((b >> 23) & 0xff) + 896) << 20) | ((b >> 3) & 0xfffff);
  return __hiloint2double(hi, (int)((unsigned)b << 29));
}

template <typename T> __device__ __forceinline__ T rsqrt_t(T x);
template <> __device__ __forceinline__ double rsqrt_t<double>(double x) { return rsqrt_d(x); }
template <> __device__ __forceinline__ float rsqrt_t<float>(float x) { return rsqrtf(x); }

// Nearest integer j of x (0 <= x < 2^22), returned as j and as the exact
// floating-point value of j: adding 1.5 * 2^52 (1.5 * 2^23 for float) leaves j in
// the low mantissa bits of the sum, with no float<->int conversion instruction.
__device__ __forceinline__ double round_node(double x, int& j) {
  const double r = x + 6755399441055744.0;
  j = __double2loint(r);
  return r - 6755399441055744.0;
}
__device__ __forceinline__ float round_node(float x, int& j) {
  const float r = x + 12582912.0f;
  j = __float_as_int(r) - 0x4B400000;
  return r - 12582912.0f;
}

template <typename T> __device__ __forceinline__ T fma_t(T a, T b, T c);
__device__ __forceinline__ double fabs_t(double x) { return fabs(x); }
__device__ __forceinline__ float fabs_t(float x) { return fabsf(x); }
__device__ __forceinline__ double fmax_t(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float fmax_t(float a, float b) { return fmaxf(a, b); }
template <> __device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }

// F_0..F_L(T) from the table by Taylor expansion about the nearest node;
// asymptotic form F_0 = sqrt(pi/T)/2, F_m = F_(m-1) (2m-1)/(2T) beyond TMAX.
template <typename T, int L> struct BoysCfg;
template <int L> struct BoysCfg<double, L> {
  static constexpr double H = BOYS64_H, TMAX = BOYS64_TMAX;
  static constexpr int NT = BOYS64_NTERM;
};
template <int L> struct BoysCfg<float, L> {
  static constexpr float H = BOYS32_H, TMAX = BOYS32_TMAX;
  static constexpr int NT = BOYS32_NTERM;
};

// Tables used by the J/K and gradient kernels, one block per order L = 0..BOYSH_LMAX:
// row j of block L holds G[k] = F_(L+k)(T_j) / k! for k < NT, then E[k] = exp(-T_j) / k!,
// so that F_L(t) = sum_k G[k] (T_j - t)^k and exp(-t) = sum_k E[k] (T_j - t)^k cost NT-1
// FMAs each.  The lower orders follow by the downward recursion
// F_m = (2t F_(m+1) + exp(-t)) / (2m + 1), whose terms are all positive.  Rows are
// 16-byte aligned and read with vector loads.
#define BOYSH_LMAX 9   // (dd|dd) gradient: L = 9
#define BOYSH64_STRIDE 16   // 6 + 6 doubles, the node T_j, padding
#define BOYSH32_STRIDE 8    // 4 + 4 floats (two 16-byte loads)
template <typename T> struct BoysHStride;
template <> struct BoysHStride<double> { static constexpr int S = BOYSH64_STRIDE, NROW = BOYS64_NROW; };
template <> struct BoysHStride<float> { static constexpr int S = BOYSH32_STRIDE, NROW = BOYS32_NROW; };

// The 2 * NT coefficients of a row (only the first NT when exp is not needed);
// FP64 rows also carry their node T_j in c[2 * NT].
template <int NT, bool EXP>
__device__ __forceinline__ void boys_row(const double* __restrict__ row, double* c) {
  const double2* v = reinterpret_cast<const double2*>(row);
#pragma unroll
  for (int i = 0; i < (EXP ? 2 * NT : NT + 1) / 2; ++i) {
    const double2 x = __ldg(v + i);
    c[2 * i] = x.x;
    c[2 * i + 1] = x.y;
  }
  const double2 x = __ldg(v + NT);   // node (and padding)
  c[2 * NT] = x.x;
}
template <int NT, bool EXP>
__device__ __forceinline__ void boys_row(const float* __restrict__ row, float* c) {
  const float4* v = reinterpret_cast<const float4*>(row);
#pragma unroll
  for (int i = 0; i < (EXP ? 2 * NT + 3 : NT + 3) / 4; ++i) {
    const float4 x = __ldg(v + i);
    c[4 * i] = x.x;
    c[4 * i + 1] = x.y;
    c[4 * i + 2] = x.z;
    c[4 * i + 3] = x.w;
  }
}

template <typename T, int L>
__device__ __forceinline__ void boys_eval(T t, const T* __restrict__ tab, T* F) {
  using C = BoysCfg<T, L>;
  static_assert(L <= BOYSH_LMAX, "the Boys tables hold orders up to BOYSH_LMAX");
  // Node index and range test in FP32 for FP64 arguments (t truncated to float by
  // moving its exponent and mantissa bits; |t - T_j| stays within 0.0126), so the
  // FP64 pipe only does dx = T_j - t.
  bool in_table;
  int j;
  T node;
  if constexpr (sizeof(T) == 8) {
    const int hi = __double2hiint(t);
    const float tf = hi < 0x38100000 ? 0.0f : __int_as_float((hi - 0x38000000) << 3);
    in_table = tf < float(C::TMAX);
    round_node(tf * float(1.0 / C::H), j);
    node = T(0);
  } else {
    in_table = t < T(C::TMAX);
    node = round_node(t * T(1.0 / C::H), j);
  }
  if (in_table) {
    const T* row = tab + ((size_t)L * BoysHStride<T>::NROW + j) * BoysHStride<T>::S;
    constexpr int NT = C::NT;
    T c[2 * NT + 4];
    boys_row<NT, (L >= 1)>(row, c);
    T dx;   // = -(t - T_j)
    if constexpr (sizeof(T) == 8) dx = c[2 * NT] - t;
    else dx = node * T(C::H) - t;
    T s = c[NT - 1];
#pragma unroll
    for (int k = NT - 2; k >= 0; --k) s = fma_t(s, dx, c[k]);
    F[L] = s;
    if constexpr (L >= 1) {
      T e = c[2 * NT - 1];
#pragma unroll
      for (int k = NT - 2; k >= 0; --k) e = fma_t(e, dx, c[NT + k]);
      const T t2 = t + t;
#pragma unroll
      for (int m = L - 1; m >= 0; --m) F[m] = fma_t(t2, F[m + 1], e) * T(1.0 / (2 * m + 1));
    }
  } else {
    const T r = rsqrt_t(t);
    F[0] = T(0.886226925452758) * r;
    const T h = T(0.5) * r * r;
#pragma unroll
    for (int m = 1; m <= L; ++m) F[m] = F[m - 1] * T(2 * m - 1) * h;
  }
}

// Error codes written by kernels into the context's device status word.
#define GBHF_DEV_ERR_TIMEOUT 1
#define GBHF_DEV_ERR_NOTCONV 2
#define GBHF_DEV_ERR_BOUNDS 4
