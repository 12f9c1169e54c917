// Symmetric eigen-solve by Householder tridiagonalisation, bisection and
// inverse iteration: eigenSolve (NumericalTools/EigenValues.hs:29-31; the
// reference calls LAPACK's dsyev family through hmatrix eigSH'), ascending
// eigenvalues with the eigenvectors as columns (sortEigenData,
// NumericalTools/VectorTools.hs:27-31).
//
// 1. k_sytrd: one CTA reduces A to tridiagonal T = Q^T A Q with the packed
//    lower triangle of A in shared memory (n <= TRIDIAG_MAX_N), n - 2
//    Householder reflectors H_k = I - tau_k v_k v_k^T (v_k[k+1] = 1).
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
#include <cfloat>

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

// Unreduced blocks: e_i is dropped when e_i^2 <= eps^2 |d_i d_(i+1)| (or is
// zero).  blk[i] = first row of row i's block, blk[n + i] = its last row.
// scal = {||T|| bound, pivmin}.
__global__ void k_tri_prep(int n, const double* __restrict__ d, double* __restrict__ e, int* __restrict__ blk,
                           double* __restrict__ scal) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double tn = 0.0, emax2 = 0.0;
  for (int i = 0; i < n; ++i) {
    double r = fabs(d[i]);
    if (i > 0) r += fabs(e[i - 1]);
    if (i + 1 < n) r += fabs(e[i]);
    tn = fmax(tn, r);
  }
  int s = 0;
  for (int i = 0; i < n; ++i) {
    bool split = (i + 1 == n);
    if (!split) {
      const double ee = e[i] * e[i];
      if (e[i] == 0.0 || ee <= kEps * kEps * fabs(d[i] * d[i + 1])) {
        e[i] = 0.0;
        split = true;
      } else {
        emax2 = fmax(emax2, ee);
      }
    }
    if (split) {
      for (int r = s; r <= i; ++r) {
        blk[r] = s;
        blk[n + r] = i;
      }
      s = i + 1;
    }
  }
  scal[0] = fmax(tn, DBL_MIN);
  scal[1] = DBL_MIN * fmax(1.0, emax2);
}

// Eigenvalues of T - x I below zero in the block [s, t] (Sturm count).
__device__ int sturm_count(const double* __restrict__ d, const double* __restrict__ e, int s, int t, double x,
                           double pivmin) {
  double q = d[s] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  int c = q < 0.0;
  for (int i = s + 1; i <= t; ++i) {
    const double ei = e[i - 1];
    q = (d[i] - x) - ei * ei / q;
    if (fabs(q) < pivmin) q = -pivmin;
    c += q < 0.0;
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
  for (int i = lane; i < m; i += 32) x[i] = start_value(seed, i);
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
        x[i] = v / u0[i];
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

// One warp per eigenvalue index k (the k-th row's block, local index k - s).
// Zt row k receives the vector (zeros outside the block), lam[k] the value.
__global__ void k_tri_vec(int n, const double* __restrict__ d, const double* __restrict__ e,
                          const int* __restrict__ blk, const double* __restrict__ scal, double* __restrict__ lam,
                          double* __restrict__ Zt) {
  extern __shared__ double smw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int k = blockIdx.x * (blockDim.x >> 5) + wib;
  if (k >= n) return;   // whole warps leave together
  double* w = smw + (long)wib * 6 * n;
  const int s = blk[k], t = blk[n + k], j = k - s;
  const double tnorm = scal[0], pivmin = scal[1];
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
  // invariant: count(lo) <= j < count(hi)
  for (int it = 0; it < 40; ++it) {
    if (hi - lo <= 2.0 * kEps * fmax(fabs(lo), fabs(hi)) + 0.5 * kEps * tb + pivmin) break;
    const double x = lo + (hi - lo) * ((double)(lane + 1) / 33.0);
    const int c = sturm_count(d, e, s, t, x, pivmin);
    const unsigned le = __ballot_sync(0xffffffffu, c <= j);
    const int lo_lane = le ? 31 - __clz(le) : -1;             // highest lane with count <= j
    const unsigned gt = ~le;
    const int hi_lane = gt ? __ffs(gt) - 1 : 32;              // lowest lane with count > j
    const double xlo = __shfl_sync(0xffffffffu, x, lo_lane < 0 ? 0 : lo_lane);
    const double xhi = __shfl_sync(0xffffffffu, x, hi_lane > 31 ? 31 : hi_lane);
    const double nlo = lo_lane >= 0 ? xlo : lo;
    double nhi = hi_lane <= 31 ? xhi : hi;
    if (!(nhi > nlo)) {   // counts not monotone in rounding: keep a valid bracket
      nhi = (lo_lane >= 0 && lo_lane < 31) ? __shfl_sync(0xffffffffu, x, lo_lane + 1) : hi;
    }
    lo = nlo;
    hi = fmax(nhi, nlo);
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

// One warp per vector (row k of Zt): z <- H_0 ... H_(n-3) z, written to column
// rank[k] of evecs (n x n row-major).
__global__ void k_tri_back(int n, const double* __restrict__ Vt, const double* __restrict__ tau,
                           const double* __restrict__ Zt, const int* __restrict__ rank, double* __restrict__ evecs) {
  extern __shared__ double smw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int k = blockIdx.x * (blockDim.x >> 5) + wib;
  if (k >= n) return;
  double* z = smw + (long)wib * n;
  for (int i = lane; i < n; i += 32) z[i] = Zt[(long)k * n + i];
  __syncwarp();
  for (int r = n - 3; r >= 0; --r) {
    const double tr = tau[r];
    if (tr == 0.0) continue;
    const double* v = Vt + (long)r * n;
    double dot = 0.0;
    for (int i = r + 1 + lane; i < n; i += 32) dot += v[i] * z[i];
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    const double f = tr * dot;
    for (int i = r + 1 + lane; i < n; i += 32) z[i] -= f * v[i];
    __syncwarp();
  }
  const int col = rank[k];
  for (int i = lane; i < n; i += 32) evecs[(long)i * n + col] = z[i];
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
  k_sytrd<<<1, 1024, smem, c->stream>>>(n, d_A, w.d.p, w.e.p, w.tau.p, w.Vt.p);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_sytrd launch");
  k_tri_prep<<<1, 32, 0, c->stream>>>(n, w.d.p, w.e.p, w.blk.p, w.scal.p);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_tri_prep launch");
  const int wpb = 2;   // warps per block: vectors spread over many SMs
  const size_t vsm = (size_t)wpb * 6 * n * sizeof(double);
  k_tri_vec<<<(n + wpb - 1) / wpb, 32 * wpb, vsm, c->stream>>>(n, w.d.p, w.e.p, w.blk.p, w.scal.p, w.lam.p,
                                                               w.Zt.p);
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
  const int bpb = 4;
  k_tri_back<<<(n + bpb - 1) / bpb, 32 * bpb, (size_t)bpb * n * sizeof(double), c->stream>>>(n, w.Vt.p, w.tau.p,
                                                                                             zin, w.rank.p, d_evecs);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_tri_back launch");
  return GBHF_OK;
}

}  // namespace gbhf
