// Symmetric eigen-solve by Householder tridiagonalisation, bisection and
// inverse iteration: eigenSolve (NumericalTools/EigenValues.hs:29-31; the
// reference calls LAPACK's dsyev family through hmatrix eigSH'), ascending
// eigenvalues with the eigenvectors as columns (sortEigenData,
// NumericalTools/VectorTools.hs:27-31).
//
// 1. k_sytrd_cluster: an 8-CTA thread-block cluster reduces A to tridiagonal
//    T = Q^T A Q with the packed lower triangle of A spread over the CTAs'
//    shared memory (k_sytrd: the same in one CTA, where clusters are not
//    available), n - 2 Householder reflectors H_k = I - tau_k v_k v_k^T
//    (v_k[k+1] = 1); n <= TRIDIAG_MAX_N.
// 2. k_tri_prep: split T into unreduced blocks at negligible off-diagonals.
// 3. k_tri_vec: one warp per eigenvalue: 32-point multisection with Sturm
//    counts on its block, then inverse iteration (LU with partial pivoting of
//    T - lambda I in shared memory) from a fixed pseudo-random start.
// 4. k_tri_fix: eigenvalues closer than 1e-11 ||T|| within a block get their
//    vectors again by inverse iteration orthogonalised against the earlier
//    ones at every step; global ascending rank of every eigenvalue.
// 5. Two Newton-Schulz steps Z <- Z (3 I - Z^T Z) / 2 on the DMMA GEMM make
//    the vectors orthonormal to rounding (inverse-iteration vectors of close
//    eigenvalues are orthogonal only to eps ||T|| / gap).
// 6. k_tri_back: one warp per vector applies H_0 ... H_(n-3) and writes the
//    vector into the column of its rank.
#include <algorithm>
#include <cfloat>

#include <cooperative_groups.h>

#include "dense.cuh"
#include "gbhf_internal.h"

namespace gbhf {

namespace {

constexpr double kEps = DBL_EPSILON;

__host__ __device__ __forceinline__ long pidx(int i, int j) { return (long)i * (i + 1) / 2 + j; }   // j <= i

// One CTA of 1024 threads.  Shared memory: packed lower triangle of A
// (n(n+1)/2), v (n), p / w (n).  Outputs: d (n), e (n - 1), tau (n), Vt (row k:
// reflector k, zero up to column k, 1 at column k + 1; rows 0 .. n - 3).
__global__ void __launch_bounds__(1024) k_sytrd(int n, const double* __restrict__ A, double* __restrict__ d,
                                                double* __restrict__ e, double* __restrict__ tau,
                                                double* __restrict__ Vt) {
  extern __shared__ double sm[];
  double* P = sm;
  double* sv = P + pidx(n, 0);   // n(n+1)/2 doubles before it
  double* sp = sv + n;
  __shared__ double s_bc[4];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (long q = tid; q < (long)n * n; q += nt) {
    const int i = (int)(q / n), j = (int)(q % n);
    if (j <= i) P[pidx(i, j)] = A[q];
  }
  __syncthreads();
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - 1 - k;   // trailing size, >= 2
    // Householder vector of column k below the diagonal
    double s = 0.0;
    for (int i = k + 2 + tid; i < n; i += nt) {
      const double x = P[pidx(i, k)];
      s += x * x;
    }
    s = block_reduce(s, false);
    if (tid == 0) {
      const double alpha = P[pidx(k + 1, k)];
      double beta = alpha, t = 0.0, scale = 0.0;
      if (s > 0.0) {
        beta = -copysign(sqrt(alpha * alpha + s), alpha);
        t = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      d[k] = P[pidx(k, k)];
      e[k] = beta;
      tau[k] = t;
      s_bc[0] = t;
      s_bc[1] = scale;
    }
    __syncthreads();
    const double t = s_bc[0], scale = s_bc[1];
    for (int i = tid; i < n; i += nt) {
      double v = 0.0;
      if (i == k + 1) v = 1.0;
      else if (i > k + 1) v = P[pidx(i, k)] * scale;
      sv[i] = v;
      Vt[(long)k * n + i] = v;
    }
    __syncthreads();
    if (t == 0.0) continue;   // uniform: s_bc is shared
    // p = t A22 v, G threads per row (G a power of two, G * m <= 1024)
    int G = 32;
    while (G > 1 && G * m > nt) G >>= 1;
    {
      const int row = k + 1 + tid / G, g = tid % G;
      double acc = 0.0;
      if (row < n) {
        for (int j = k + 1 + g; j < n; j += G) {
          const double a = j <= row ? P[pidx(row, j)] : P[pidx(j, row)];
          acc += a * sv[j];
        }
      }
      for (int o = G >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (row < n && g == 0) sp[row] = t * acc;
    }
    __syncthreads();
    // w = p - (t/2)(p.v) v
    double pv = 0.0;
    for (int i = k + 1 + tid; i < n; i += nt) pv += sp[i] * sv[i];
    pv = block_reduce(pv, false);
    if (tid == 0) s_bc[2] = -0.5 * t * pv;
    __syncthreads();
    const double c2 = s_bc[2];
    for (int i = k + 1 + tid; i < n; i += nt) sp[i] += c2 * sv[i];
    __syncthreads();
    // A22 -= v w^T + w v^T on the packed trailing triangle: local rows r and
    // m - 1 - r share a group (r + 1 + m - r = m + 1 elements per pair)
    {
      const int npair = (m + 1) / 2;
      int G2 = 32;
      while (G2 > 1 && G2 * npair > nt) G2 >>= 1;
      const int q = tid / G2, g = tid % G2;
      if (q < npair) {
        const int r1 = q, r2 = m - 1 - q;
        const int len = (r1 + 1) + (r2 != r1 ? r2 + 1 : 0);
        for (int u = g; u < len; u += G2) {
          int r, cidx;
          if (u <= r1) {
            r = r1;
            cidx = u;
          } else {
            r = r2;
            cidx = u - r1 - 1;
          }
          const int i = k + 1 + r, j = k + 1 + cidx;
          P[pidx(i, j)] -= sv[i] * sp[j] + sp[i] * sv[j];
        }
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (n >= 2) {
      d[n - 2] = P[pidx(n - 2, n - 2)];
      e[n - 2] = P[pidx(n - 1, n - 2)];
      tau[n - 2] = 0.0;
    }
    d[n - 1] = P[pidx(n - 1, n - 1)];
    tau[n - 1] = 0.0;
  }
}

// The same reduction by one thread-block cluster of SY_CS CTAs: CTA r owns
// the rows i = r (mod SY_CS) of the packed lower triangle in its shared memory,
// so the FP64 work of a step is split SY_CS ways.  Per step k, two cluster
// barriers:
//   A. every CTA pushes its entries x_i = A_ik (i > k) into every CTA's copy of
//      the Householder vector and its partial |x|^2 into its own slot; after
//      the barrier each CTA sums the partials in rank order (all CTAs get the
//      same bits), forms tau and scales its copy into v;
//   B. p_part[j] = sum over its own rows i > j of A_ij v_i (+ the row dot
//      sum_(l <= j) A_jl v_l for its own rows j); after the barrier every CTA
//      sums p_j over the ranks (rank order), forms p.v and w = p - (tau/2)(p.v) v
//      for all j, and updates its own rows A_il -= v_i w_l + w_i v_l.
// The Householder vector and the partial slots alternate between two buffers
// by step parity (a CTA writes step k + 1's values into another CTA's memory
// while that CTA may still read step k's).  Outputs as k_sytrd.
constexpr int SY_CS = 8, SY_THREADS = 512;

__host__ __device__ __forceinline__ long sy_off(int r, int q) {   // start of local row q of rank r
  return (long)q * (r + 1) + (long)SY_CS * q * (q - 1) / 2;
}
__host__ __device__ __forceinline__ long sy_local_doubles(int n, int r) {
  const int nq = n > r ? (n - r + SY_CS - 1) / SY_CS : 0;
  return sy_off(r, nq);
}

__global__ void __cluster_dims__(SY_CS, 1, 1) __launch_bounds__(SY_THREADS)
    k_sytrd_cluster(int n, const double* __restrict__ A, double* __restrict__ d, double* __restrict__ e,
                    double* __restrict__ tau, double* __restrict__ Vt) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ double sm[];
  const int r = (int)cluster.block_rank(), tid = threadIdx.x, nt = blockDim.x;
  const int nq = n > r ? (n - r + SY_CS - 1) / SY_CS : 0;   // rows owned
  // The buffers other CTAs reach come first, at the same offsets in every CTA
  // (a remote address is the local offset mapped into the other CTA's window);
  // the owned rows, whose size depends on the rank, follow them.
  double* sv = sm;                   // 2 x n: Householder vector, by step parity
  double* sw = sv + 2 * n;           // n: p, then w
  double* pp = sw + n;               // n: this CTA's partial p
  double* red = pp + n;              // 2 x 4: partial |x|^2 by step parity
  double* P = red + 8;               // owned rows, packed
  __shared__ double s_bc[4];
  __shared__ double s_red[SY_THREADS / 32];
  auto row_of = [&](int q) { return r + SY_CS * q; };
  auto bsum = [&](double v) -> double {   // block sum, valid in every thread
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((tid & 31) == 0) s_red[tid >> 5] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nt / 32; ++w) t += s_red[w];
    return t;
  };
  for (int q = 0; q < nq; ++q) {
    const int i = row_of(q);
    for (int j = tid; j <= i; j += nt) P[sy_off(r, q) + j] = A[(long)i * n + j];
  }
  cluster.sync();
  for (int k = 0; k + 2 < n; ++k) {
    const int par = k & 1;
    double* v = sv + par * n;
    // A: push x_i = A_ik (i > k) of own rows into every CTA's copy; partial |x|^2 (i > k + 1)
    const int q0 = (k + 1 - r + SY_CS - 1) / SY_CS > 0 ? (k + 1 - r + SY_CS - 1) / SY_CS : 0;   // first own row > k
    double s = 0.0;
    for (int idx = tid; idx < (nq - q0) * SY_CS; idx += nt) {
      const int q = q0 + idx / SY_CS, dst = idx % SY_CS;
      const int i = row_of(q);
      const double x = P[sy_off(r, q) + k];
      double* rv = cluster.map_shared_rank(v, dst);
      rv[i] = x;
      if (dst == 0 && i > k + 1) s += x * x;
    }
    s = bsum(s);
    if (tid == 0) red[par * 4] = s;
    if (k % SY_CS == r && tid == 0) d[k] = P[sy_off(r, k / SY_CS) + k];
    cluster.sync();
    if (tid < 32) {
      // the SY_CS partials read at once (one remote latency), summed in rank order
      const double part = tid < SY_CS ? *cluster.map_shared_rank(red + par * 4, tid) : 0.0;
      double tot = 0.0;
#pragma unroll
      for (int rr = 0; rr < SY_CS; ++rr) tot += __shfl_sync(0xffffffffu, part, rr);
      const double alpha = v[k + 1];
      double beta = alpha, t = 0.0, scale = 0.0;
      if (tot > 0.0) {
        beta = -copysign(sqrt(alpha * alpha + tot), alpha);
        t = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      if (r == 0 && tid == 0) {
        e[k] = beta;
        tau[k] = t;
      }
      if (tid == 0) {
        s_bc[0] = t;
        s_bc[1] = scale;
      }
    }
    __syncthreads();
    const double t = s_bc[0], scale = s_bc[1];
    for (int i = k + 1 + tid; i < n; i += nt) v[i] = i == k + 1 ? 1.0 : v[i] * scale;
    __syncthreads();
    for (int q = tid; q < nq; q += nt) {   // own entries of Vt row k
      const int i = row_of(q);
      Vt[(long)k * n + i] = i <= k ? 0.0 : v[i];
    }
    // (with t = 0 the steps below leave A unchanged; they still run, so that
    // every CTA passes the same barriers whatever its data)
    // B: partial p (column part over own rows i > j, then the row dots of own rows)
    for (int j = k + 1 + tid; j < n; j += nt) {
      double acc = 0.0;
      for (int q = (j + 1 - r + SY_CS - 1) / SY_CS > 0 ? (j + 1 - r + SY_CS - 1) / SY_CS : 0; q < nq; ++q)
        acc += P[sy_off(r, q) + j] * v[row_of(q)];
      pp[j] = acc;
    }
    __syncthreads();
    {
      const int nown = nq - q0;                 // own rows > k
      int G = 32;
      while (G > 1 && G * nown > nt) G >>= 1;
      const int qi = q0 + tid / G, g = tid % G;
      double acc = 0.0;
      if (tid / G < nown) {
        const long off = sy_off(r, qi);
        for (int l = k + 1 + g; l <= row_of(qi); l += G) acc += P[off + l] * v[l];
      }
      for (int o = G >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (tid / G < nown && g == 0) pp[row_of(qi)] += acc;
    }
    cluster.sync();
    // p_j = t sum_r pp_r[j] for every j; p.v; w
    double pv = 0.0;
    for (int j = k + 1 + tid; j < n; j += nt) {
      double part[SY_CS];
#pragma unroll
      for (int rr = 0; rr < SY_CS; ++rr) part[rr] = cluster.map_shared_rank(pp, rr)[j];
      double acc = 0.0;
#pragma unroll
      for (int rr = 0; rr < SY_CS; ++rr) acc += part[rr];
      const double p = t * acc;
      sw[j] = p;
      pv += p * v[j];
    }
    pv = bsum(pv);
    const double c2 = -0.5 * t * pv;
    for (int j = k + 1 + tid; j < n; j += nt) sw[j] += c2 * v[j];
    __syncthreads();
    // own rows: A_il -= v_i w_l + w_i v_l, l in (k, i]
    {
      const int nown = nq - q0;
      int G = 32;
      while (G > 1 && G * nown > nt) G >>= 1;
      const int qi = q0 + tid / G, g = tid % G;
      if (tid / G < nown) {
        const int i = row_of(qi);
        const long off = sy_off(r, qi);
        const double vi = v[i], wi = sw[i];
        for (int l = k + 1 + g; l <= i; l += G) P[off + l] -= vi * sw[l] + wi * v[l];
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (n >= 2) {
      if ((n - 2) % SY_CS == r) d[n - 2] = P[sy_off(r, (n - 2) / SY_CS) + (n - 2)];
      if ((n - 1) % SY_CS == r) e[n - 2] = P[sy_off(r, (n - 1) / SY_CS) + (n - 2)];
      if (r == 0) tau[n - 2] = 0.0;
    }
    if ((n - 1) % SY_CS == r) d[n - 1] = P[sy_off(r, (n - 1) / SY_CS) + (n - 1)];
    if (r == 0) tau[n - 1] = 0.0;
  }
  cluster.sync();   // no CTA leaves while another may still read its shared memory
}

// Unreduced blocks: e_i is dropped when e_i^2 <= eps^2 |d_i d_(i+1)| (or is
// zero).  blk[i] = first row of row i's block, blk[n + i] = its last row.
// Also e2 = e^2, and single-precision copies df = d, e2f = e^2 for the coarse
// bisection.  scal = {||T|| bound, pivmin, single-precision pivmin}.  One block
// of 256 threads; d and e are staged in shared memory (n <= 1024).
__global__ void __launch_bounds__(256) k_tri_prep(int n, const double* __restrict__ d, double* __restrict__ e,
                                                  int* __restrict__ blk, double* __restrict__ e2,
                                                  float* __restrict__ df, float* __restrict__ e2f,
                                                  double* __restrict__ scal) {
  __shared__ double sd[1024], se[1024];
  __shared__ double s_red[8];
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += blockDim.x) {
    sd[i] = d[i];
    se[i] = i + 1 < n ? e[i] : 0.0;
  }
  __syncthreads();
  double tn = 0.0;
  for (int i = tid; i < n; i += blockDim.x) {
    double r = fabs(sd[i]);
    if (i > 0) r += fabs(se[i - 1]);
    if (i + 1 < n) r += fabs(se[i]);
    tn = fmax(tn, r);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
  if ((tid & 31) == 0) s_red[tid >> 5] = tn;
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) tn = fmax(tn, s_red[w]);
    double emax2 = 0.0;
    int s0 = 0;
    for (int i = 0; i < n; ++i) {
      bool split = (i + 1 == n);
      if (!split) {
        const double ee = se[i] * se[i];
        if (se[i] == 0.0 || ee <= kEps * kEps * fabs(sd[i] * sd[i + 1])) {
          se[i] = 0.0;
          split = true;
        } else {
          emax2 = fmax(emax2, ee);
        }
      }
      if (split) {
        for (int r = s0; r <= i; ++r) {
          blk[r] = s0;
          blk[n + r] = i;
        }
        s0 = i + 1;
      }
    }
    scal[0] = fmax(tn, DBL_MIN);
    scal[1] = DBL_MIN * fmax(1.0, emax2);
    scal[2] = (double)FLT_MIN * fmax(1.0, emax2);
  }
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) {
    const double ee = se[i] * se[i];
    if (i + 1 < n) e[i] = se[i];
    e2[i] = ee;
    df[i] = (float)sd[i];
    e2f[i] = (float)ee;
  }
}

// 1/q by one Newton-Raphson step, r1 = r0 + r0 (1 - q r0), from the
// single-precision reciprocal (relative error ~2^-46); outside the single-
// precision range the plain quotient.  Only the sign of each pivot of a Sturm
// sequence matters, so this accuracy is ample.
__device__ __forceinline__ double recip_nr(double q) {
  const double aq = fabs(q);
  if (!(aq > 1e-30 && aq < 1e30)) return 1.0 / q;
  const double r0 = (double)__frcp_rn((float)q);
  return fma(r0, fma(-q, r0, 1.0), r0);
}

// Eigenvalues of T - x I below zero in the block [s, t] (Sturm count); e2 = e^2.
__device__ int sturm_count(const double* __restrict__ d, const double* __restrict__ e2, int s, int t, double x,
                           double pivmin) {
  double q = d[s] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  int c = q < 0.0;
  for (int i = s + 1; i <= t; ++i) {
    q = (d[i] - x) - e2[i - 1] * recip_nr(q);
    if (fabs(q) < pivmin) q = -pivmin;
    c += q < 0.0;
  }
  return c;
}

// The same in single precision (coarse bracketing only).
__device__ int sturm_count_f(const float* __restrict__ d, const float* __restrict__ e2, int s, int t, float x,
                             float pivmin) {
  float q = d[s] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  int c = q < 0.0f;
  for (int i = s + 1; i <= t; ++i) {
    q = (d[i] - x) - __fdividef(e2[i - 1], q);
    if (fabsf(q) < pivmin) q = -pivmin;
    c += q < 0.0f;
  }
  return c;
}

// Pseudo-random start in (-1, 1) for vector k, element i (a fixed integer hash).
__device__ __forceinline__ double start_value(int k, int i) {
  unsigned h = (unsigned)k * 0x9E3779B1u ^ ((unsigned)i + 0x7F4A7C15u) * 0x85EBCA77u;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return ((double)(h >> 8) + 0.5) * (2.0 / 16777216.0) - 1.0;
}

// Inverse iteration for eigenvalue lam of block [s, t] (m = t - s + 1 >= 2),
// executed by one warp.  w: 6 m doubles of this warp's shared memory.  The
// result (unit norm) goes to zrow[s .. t]; with nprev > 0 every iterate is
// orthogonalised against rows prev[0 .. nprev) (global rows of the same
// block, unit norm) first.
__device__ void inverse_iteration(const double* __restrict__ d, const double* __restrict__ e, int s, int t,
                                  double lam, double tnorm, int seed, double* w, double* __restrict__ zrow,
                                  const double* __restrict__ prev, long prev_stride, int nprev) {
  const int lane = threadIdx.x & 31;
  const int m = t - s + 1;
  double* u0 = w;
  double* u1 = w + m;
  double* u2 = w + 2 * m;
  double* l = w + 3 * m;   // multiplier; sign bit of the pivot flag kept in piv
  double* piv = w + 4 * m;
  double* x = w + 5 * m;
  const double eps_piv = kEps * tnorm;
  if (lane == 0) {
    // current row (r0, r1) at columns (i, i + 1)
    double r0 = d[s] - lam, r1 = e[s];
    for (int i = 0; i + 1 < m; ++i) {
      const double sub = e[s + i], nd = d[s + i + 1] - lam, ns1 = (i + 2 < m) ? e[s + i + 1] : 0.0;
      if (fabs(r0) >= fabs(sub)) {
        if (r0 == 0.0) r0 = eps_piv;
        const double mlt = sub / r0;
        u0[i] = r0;
        u1[i] = r1;
        u2[i] = 0.0;
        l[i] = mlt;
        piv[i] = 0.0;
        r0 = nd - mlt * r1;
        r1 = ns1;
      } else {
        const double mlt = r0 / sub;
        u0[i] = sub;
        u1[i] = nd;
        u2[i] = ns1;
        l[i] = mlt;
        piv[i] = 1.0;
        r0 = r1 - mlt * nd;
        r1 = -mlt * ns1;
      }
    }
    if (r0 == 0.0) r0 = eps_piv;
    u0[m - 1] = r0;
  }
  __syncwarp();
  // u0 now holds the pivots' reciprocals (one division each, across the lanes)
  for (int i = lane; i < m; i += 32) {
    u0[i] = 1.0 / u0[i];
    x[i] = start_value(seed, i);
  }
  __syncwarp();
  for (int it = 0; it < 4; ++it) {
    if (lane == 0) {
      for (int i = 0; i + 1 < m; ++i) {
        if (piv[i] != 0.0) {
          const double tmp = x[i];
          x[i] = x[i + 1];
          x[i + 1] = tmp;
        }
        x[i + 1] -= l[i] * x[i];
      }
      for (int i = m - 1; i >= 0; --i) {
        double v = x[i];
        if (i + 1 < m) v -= u1[i] * x[i + 1];
        if (i + 2 < m) v -= u2[i] * x[i + 2];
        x[i] = v * u0[i];
      }
    }
    __syncwarp();
    for (int p = 0; p < nprev; ++p) {
      const double* pr = prev + p * prev_stride + s;
      double dot = 0.0;
      for (int i = lane; i < m; i += 32) dot += pr[i] * x[i];
      for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
      for (int i = lane; i < m; i += 32) x[i] -= dot * pr[i];
      __syncwarp();
    }
    double nrm = 0.0;
    for (int i = lane; i < m; i += 32) nrm += x[i] * x[i];
    for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
    const double inv = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    for (int i = lane; i < m; i += 32) x[i] *= inv;
    __syncwarp();
  }
  for (int i = lane; i < m; i += 32) zrow[s + i] = x[i];
  __syncwarp();
}

// One step of 32-point multisection: the new bracket from the counts at the
// 32 interior points x (one per lane); invariant count(lo) <= j < count(hi).
template <typename R>
__device__ __forceinline__ void multisect(R x, int c, int j, R& lo, R& hi) {
  const unsigned le = __ballot_sync(0xffffffffu, c <= j);
  const int lo_lane = le ? 31 - __clz(le) : -1;             // highest lane with count <= j
  const unsigned gt = ~le;
  const int hi_lane = gt ? __ffs(gt) - 1 : 32;              // lowest lane with count > j
  const R xlo = __shfl_sync(0xffffffffu, x, lo_lane < 0 ? 0 : lo_lane);
  const R xhi = __shfl_sync(0xffffffffu, x, hi_lane > 31 ? 31 : hi_lane);
  const R nlo = lo_lane >= 0 ? xlo : lo;
  R nhi = hi_lane <= 31 ? xhi : hi;
  if (!(nhi > nlo)) {   // counts not monotone in rounding: keep a valid bracket
    const R xn = __shfl_sync(0xffffffffu, x, (lo_lane >= 0 && lo_lane < 31) ? lo_lane + 1 : 31);
    nhi = (lo_lane >= 0 && lo_lane < 31) ? xn : hi;
  }
  lo = nlo;
  hi = nhi > nlo ? nhi : nlo;
}

// One warp per eigenvalue index k (the k-th row's block, local index k - s).
// Zt row k receives the vector (zeros outside the block), lam[k] the value.
// The bracket is first narrowed to ~1e-4 of the block's Gershgorin bound with
// single-precision Sturm counts (64 times the FP64 rate on this GPU), widened
// by a margin well above their error, checked with two FP64 counts (else the
// whole interval is kept), then refined in FP64.
__global__ void k_tri_vec(int n, const double* __restrict__ d, const double* __restrict__ e,
                          const double* __restrict__ e2, const float* __restrict__ df,
                          const float* __restrict__ e2f, const int* __restrict__ blk,
                          const double* __restrict__ scal, double* __restrict__ lam, double* __restrict__ Zt) {
  extern __shared__ double smw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int k = blockIdx.x * (blockDim.x >> 5) + wib;
  if (k >= n) return;   // whole warps leave together
  double* w = smw + (long)wib * 6 * n;
  const int s = blk[k], t = blk[n + k], j = k - s;
  const double tnorm = scal[0], pivmin = scal[1];
  const float pivf = (float)scal[2];
  double* zrow = Zt + (long)k * n;
  for (int i = lane; i < n; i += 32) zrow[i] = (i == k && s == t) ? 1.0 : 0.0;
  if (s == t) {
    if (lane == 0) lam[k] = d[k];
    return;
  }
  // Gershgorin interval of the block
  double lo = INFINITY, hi = -INFINITY;
  for (int i = s + lane; i <= t; i += 32) {
    const double r = (i > s ? fabs(e[i - 1]) : 0.0) + (i < t ? fabs(e[i]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const double tb = fmax(fabs(lo), fabs(hi));
  lo -= 2.0 * kEps * tb + 2.0 * pivmin;
  hi += 2.0 * kEps * tb + 2.0 * pivmin;
  {
    // coarse: three FP32 rounds (width / 33^3), then a margin of 2e-4 tb on each side
    float lof = (float)lo, hif = (float)hi;
    for (int it = 0; it < 3; ++it) {
      const float x = lof + (hif - lof) * ((float)(lane + 1) / 33.0f);
      multisect<float>(x, sturm_count_f(df, e2f, s, t, x, pivf), j, lof, hif);
    }
    const double lo2 = fmax(lo, (double)lof - 2e-4 * tb), hi2 = fmin(hi, (double)hif + 2e-4 * tb);
    int cv = 0;
    if (lane < 2) cv = sturm_count(d, e2, s, t, lane == 0 ? lo2 : hi2, pivmin);
    const int c_lo = __shfl_sync(0xffffffffu, cv, 0), c_hi = __shfl_sync(0xffffffffu, cv, 1);
    if (c_lo <= j && c_hi > j) {
      lo = lo2;
      hi = hi2;
    }
  }
  for (int it = 0; it < 40; ++it) {
    if (hi - lo <= 2.0 * kEps * fmax(fabs(lo), fabs(hi)) + 0.5 * kEps * tb + pivmin) break;
    const double x = lo + (hi - lo) * ((double)(lane + 1) / 33.0);
    multisect<double>(x, sturm_count(d, e2, s, t, x, pivmin), j, lo, hi);
  }
  const double lambda = 0.5 * (lo + hi);
  if (lane == 0) lam[k] = lambda;
  inverse_iteration(d, e, s, t, lambda, tnorm, k, w, zrow, nullptr, 0, 0);
}

// One block.  Warp 0 recomputes the vectors of eigenvalues within 1e-11 ||T||
// of the previous one in the same block, orthogonalised against the earlier
// members of that run; then every thread ranks the eigenvalues (ascending,
// ties by index) and writes evals in sorted order.
__global__ void __launch_bounds__(256) k_tri_fix(int n, const double* __restrict__ d, const double* __restrict__ e,
                          const int* __restrict__ blk, const double* __restrict__ scal,
                          const double* __restrict__ lam, double* __restrict__ Zt, int* __restrict__ rank,
                          double* __restrict__ evals) {
  extern __shared__ double smw[];
  const double tnorm = scal[0];
  if (threadIdx.x < 32) {
    int run0 = 0;
    for (int k = 1; k < n; ++k) {
      const bool same = blk[k] == blk[k - 1] && blk[k] != blk[n + k];
      if (!(same && lam[k] - lam[k - 1] < 1e-11 * tnorm)) {
        run0 = k;
        continue;
      }
      inverse_iteration(d, e, blk[k], blk[n + k], lam[k], tnorm, k + 7919, smw, Zt + (long)k * n,
                        Zt + (long)run0 * n, n, k - run0);
    }
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double v = lam[k];
    int r = 0;
    for (int q = 0; q < n; ++q) {
      const double u = lam[q];
      r += (u < v) || (u == v && q < k);
    }
    rank[k] = r;
    evals[r] = v;
  }
}

__global__ void k_ns_mat(int n, const double* __restrict__ S, double* __restrict__ M) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < (long)n * n; q += (long)gridDim.x * blockDim.x) {
    const int i = (int)(q / n), j = (int)(q % n);
    M[q] = (i == j ? 1.5 : 0.0) - 0.5 * S[q];
  }
}

// z <- H_0 ... H_(n-3) z for every vector (rows of Zt), written to column
// rank[k] of evecs (n x n row-major).  One warp per vector, TB_WARPS vectors
// per block; each reflector row is loaded once per block into shared memory
// (double-buffered: row r - 1 loads while row r is applied), one barrier per
// reflector.
constexpr int TB_WARPS = 8;

__global__ void __launch_bounds__(TB_WARPS * 32) k_tri_back(int n, const double* __restrict__ Vt,
                                                            const double* __restrict__ tau,
                                                            const double* __restrict__ Zt,
                                                            const int* __restrict__ rank,
                                                            double* __restrict__ evecs) {
  extern __shared__ double smw[];
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  const int k = blockIdx.x * TB_WARPS + wib;
  double* vbuf = smw;                       // 2 x n
  double* z = smw + 2 * n + (long)wib * n;  // this warp's vector
  if (k < n)
    for (int i = lane; i < n; i += 32) z[i] = Zt[(long)k * n + i];
  const int r0 = n - 3;
  if (r0 >= 0)
    for (int i = tid; i < n; i += blockDim.x) vbuf[(r0 & 1) * n + i] = Vt[(long)r0 * n + i];
  __syncthreads();
  for (int r = r0; r >= 0; --r) {
    // next row into the other buffer (read in the step after the barrier below)
    if (r > 0)
      for (int i = tid; i < n; i += blockDim.x) vbuf[((r - 1) & 1) * n + i] = Vt[(long)(r - 1) * n + i];
    const double tr = tau[r];
    if (k < n && tr != 0.0) {
      const double* v = vbuf + (r & 1) * n;
      double dot = 0.0;
      for (int i = r + 1 + lane; i < n; i += 32) dot += v[i] * z[i];
      for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
      const double f = tr * dot;
      for (int i = r + 1 + lane; i < n; i += 32) z[i] -= f * v[i];
    }
    __syncthreads();
  }
  if (k < n) {
    const int col = rank[k];
    for (int i = lane; i < n; i += 32) evecs[(long)i * n + col] = z[i];
  }
}

}  // namespace

size_t tridiag_smem_bytes(int n) { return (size_t)(pidx(n, 0) + 2 * (long)n) * sizeof(double); }

// d_evecs (n x n): eigenvectors of A in columns, ascending eigenvalues.
gbhf_status eigh_tridiag(gbhf_ctx* c, int n, const double* d_A, double* d_evals, double* d_evecs) {
  TridiagWork& w = c->tri;
  const size_t nn = (size_t)n * n;
  GBHF_CUDA(c, w.d.alloc(n));
  GBHF_CUDA(c, w.e.alloc(n));
  GBHF_CUDA(c, w.tau.alloc(n));
  GBHF_CUDA(c, w.lam.alloc(n));
  GBHF_CUDA(c, w.scal.alloc(4));
  GBHF_CUDA(c, w.e2.alloc(n));
  GBHF_CUDA(c, w.df.alloc(n));
  GBHF_CUDA(c, w.e2f.alloc(n));
  GBHF_CUDA(c, w.Vt.alloc(nn));
  GBHF_CUDA(c, w.Zt.alloc(nn));
  GBHF_CUDA(c, w.Z2.alloc(nn));
  GBHF_CUDA(c, w.S.alloc(nn));
  GBHF_CUDA(c, w.M.alloc(nn));
  GBHF_CUDA(c, w.blk.alloc(2 * (size_t)n));
  GBHF_CUDA(c, w.rank.alloc(n));
  const size_t smem = tridiag_smem_bytes(n);
  // The attribute belongs to the kernel (per device, for the whole process):
  // always the largest size, so that no context lowers it under another's launch.
  GBHF_CUDA(c, cudaFuncSetAttribute(k_sytrd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)tridiag_smem_bytes(TRIDIAG_MAX_N)));
  if (n > 1) {
    GBHF_CUDA(c, cudaMemsetAsync(w.e.p, 0, n * sizeof(double), c->stream));
  }
  // the cluster form when the device runs an 8-CTA cluster of it (checked once)
  long sy_loc = 0;
  for (int r = 0; r < SY_CS; ++r) sy_loc = std::max(sy_loc, sy_local_doubles(n, r));
  const size_t sy_smem = (size_t)(sy_loc + 4L * n + 8) * sizeof(double);
  if (c->sytrd_cluster == 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(SY_CS);
    cfg.blockDim = dim3(SY_THREADS);
    cfg.dynamicSmemBytes = (size_t)(sy_local_doubles(TRIDIAG_MAX_N, SY_CS - 1) + 4L * TRIDIAG_MAX_N + 8) * 8;
    int ncl = 0;
    const cudaError_t ce = cudaOccupancyMaxActiveClusters(&ncl, k_sytrd_cluster, &cfg);
    c->sytrd_cluster = (ce == cudaSuccess && ncl >= 1) ? 1 : -1;
    (void)cudaGetLastError();   // a refused query leaves no error behind
  }
  if (c->sytrd_cluster > 0 && !c->force_sytrd_single && n >= 2 * SY_CS) {
    k_sytrd_cluster<<<SY_CS, SY_THREADS, sy_smem, c->stream>>>(n, d_A, w.d.p, w.e.p, w.tau.p, w.Vt.p);
    count_launch(c);
    GBHF_LAUNCHED(c, "k_sytrd_cluster launch");
  } else {
    k_sytrd<<<1, 1024, smem, c->stream>>>(n, d_A, w.d.p, w.e.p, w.tau.p, w.Vt.p);
    count_launch(c);
    GBHF_LAUNCHED(c, "k_sytrd launch");
  }
  k_tri_prep<<<1, 256, 0, c->stream>>>(n, w.d.p, w.e.p, w.blk.p, w.e2.p, w.df.p, w.e2f.p, w.scal.p);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_tri_prep launch");
  const int wpb = 2;   // warps per block: vectors spread over many SMs
  const size_t vsm = (size_t)wpb * 6 * n * sizeof(double);
  k_tri_vec<<<(n + wpb - 1) / wpb, 32 * wpb, vsm, c->stream>>>(n, w.d.p, w.e.p, w.e2.p, w.df.p, w.e2f.p, w.blk.p,
                                                               w.scal.p, w.lam.p, w.Zt.p);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_tri_vec launch");
  k_tri_fix<<<1, 256, 6 * n * sizeof(double), c->stream>>>(n, w.d.p, w.e.p, w.blk.p, w.scal.p, w.lam.p, w.Zt.p,
                                                            w.rank.p, d_evals);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_tri_fix launch");
  // Newton-Schulz: Zt <- (3 I - Zt Zt^T) Zt / 2, twice
  double* zin = w.Zt.p;
  double* zout = w.Z2.p;
  for (int step = 0; step < 2; ++step) {
    GBHF_TRY(gemm(c, false, true, n, n, n, 1.0, zin, n, zin, n, 0.0, w.S.p, n, true));
    k_ns_mat<<<std::max(1, std::min(c->nsm * 4, (int)((nn + 255) / 256))), 256, 0, c->stream>>>(n, w.S.p, w.M.p);
    count_launch(c);
    GBHF_LAUNCHED(c, "k_ns_mat launch");
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, w.M.p, n, zin, n, 0.0, zout, n));
    std::swap(zin, zout);
  }
  k_tri_back<<<(n + TB_WARPS - 1) / TB_WARPS, TB_WARPS * 32, (size_t)(2 + TB_WARPS) * n * sizeof(double),
               c->stream>>>(n, w.Vt.p, w.tau.p, zin, w.rank.p, d_evecs);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_tri_back launch");
  return GBHF_OK;
}

}  // namespace gbhf
