// Dense FP64 linear algebra for the SCF: DMMA GEMM (mma.sync m8n8k4 f64),
// cooperative parallel Jacobi eigen-solver, DIIS helpers and reductions.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gbhf_internal.h"
#include "dense.cuh"
#include "jacobi.cuh"

namespace gbhf {

// ------------------------------------------------------------------ GEMM ----
// C = alpha * op(A) * op(B) + beta * C, row-major.  op(A) is m x k (A stored
// m x k, or k x m when ta), op(B) is k x n.  CTA tile 64x64, 4 warps of 32x32,
// each warp a 4x4 grid of 8x8 DMMA tiles, k-step 16.
constexpr int GT = 64, GK = 16;


__global__ void __launch_bounds__(128) k_dgemm(bool ta, bool tb, int m, int n, int k, double alpha,
                                               const double* __restrict__ A, int lda, const double* __restrict__ B,
                                               int ldb, double beta, double* __restrict__ C, int ldc) {
  __shared__ double As[GT][GK + 1];
  __shared__ double Bs[GK][GT + 2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int row0 = blockIdx.y * GT, col0 = blockIdx.x * GT;
  const int wr = (warp >> 1) * 32, wc = (warp & 1) * 32;
  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
  for (int kk = 0; kk < k; kk += GK) {
    // A tile: 64 x 16
    for (int idx = tid; idx < GT * GK; idx += 128) {
      int r, cc;
      if (!ta) {
        r = idx / GK;
        cc = idx % GK;
      } else {
        cc = idx / GT;
        r = idx % GT;
      }
      const int gr = row0 + r, gk = kk + cc;
      double v = 0.0;
      if (gr < m && gk < k) v = ta ? A[(long)gk * lda + gr] : A[(long)gr * lda + gk];
      As[r][cc] = v;
    }
    // B tile: 16 x 64
    for (int idx = tid; idx < GK * GT; idx += 128) {
      int r, cc;
      if (!tb) {
        r = idx / GT;
        cc = idx % GT;
      } else {
        cc = idx / GK;
        r = idx % GK;
      }
      const int gk = kk + r, gc = col0 + cc;
      double v = 0.0;
      if (gk < k && gc < n) v = tb ? B[(long)gc * ldb + gk] : B[(long)gk * ldb + gc];
      Bs[r][cc] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k4 = 0; k4 < GK; k4 += 4) {
      double af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = As[wr + i * 8 + (lane >> 2)][k4 + (lane & 3)];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = Bs[k4 + (lane & 3)][wc + j * 8 + (lane >> 2)];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dmma(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = row0 + wr + i * 8 + (lane >> 2);
        const int cc = col0 + wc + j * 8 + 2 * (lane & 3) + h;
        if (r < m && cc < n) {
          double* p = C + (long)r * ldc + cc;
          *p = alpha * acc[i][j][h] + (beta == 0.0 ? 0.0 : beta * *p);
        }
      }
}

// Small-matrix variant: 32x32 C tile per CTA (4 warps of 16x16 = 2x2 DMMA
// tiles), K split over gridDim.z slices whose partial products are added
// with FP64 atomics into C (pre-scaled by beta), so that N ~ 200 matrices
// still occupy every SM.  sym (square C known to be symmetric, e.g. P P or
// X^T F X): only the tiles on and above the diagonal are computed, each
// added to its mirror position as well.
constexpr int ST = 32, SK = 16;

struct SplitSmem {
  double As[ST][SK + 1];
  double Bs[SK][ST + 2];
};

// One 32 x 32 tile (row tile rt, column tile ct) of C += alpha op(A) op(B) over
// k in [k0, k1), added with FP64 atomics; sym: also added at the mirror tile
// (rt < ct); trace (nullable): the tile's diagonal entries summed into *trace.
// Called by every thread of a 128-thread block.
__device__ __forceinline__ void dgemm_tile(bool ta, bool tb, bool sym, int m, int n, int rt, int ct, int k0, int k1,
                                           double alpha, const double* __restrict__ A, int lda,
                                           const double* __restrict__ B, int ldb, double* __restrict__ C, int ldc,
                                           double* trace, SplitSmem& sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int row0 = rt * ST, col0 = ct * ST;
  const int wr = (warp >> 1) * 16, wc = (warp & 1) * 16;
  double acc[2][2][2] = {};
  for (int kk = k0; kk < k1; kk += SK) {
    for (int idx = tid; idx < ST * SK; idx += 128) {
      int r, cc;
      if (!ta) {
        r = idx / SK;
        cc = idx % SK;
      } else {
        cc = idx / ST;
        r = idx % ST;
      }
      const int gr = row0 + r, gk = kk + cc;
      double v = 0.0;
      if (gr < m && gk < k1) v = ta ? A[(long)gk * lda + gr] : A[(long)gr * lda + gk];
      sm.As[r][cc] = v;
    }
    for (int idx = tid; idx < SK * ST; idx += 128) {
      int r, cc;
      if (!tb) {
        r = idx / ST;
        cc = idx % ST;
      } else {
        cc = idx / SK;
        r = idx % SK;
      }
      const int gk = kk + r, gc = col0 + cc;
      double v = 0.0;
      if (gk < k1 && gc < n) v = tb ? B[(long)gc * ldb + gk] : B[(long)gk * ldb + gc];
      sm.Bs[r][cc] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k4 = 0; k4 < SK; k4 += 4) {
      double af[2], bf[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) af[i] = sm.As[wr + i * 8 + (lane >> 2)][k4 + (lane & 3)];
#pragma unroll
      for (int j = 0; j < 2; ++j) bf[j] = sm.Bs[k4 + (lane & 3)][wc + j * 8 + (lane >> 2)];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) dmma(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = row0 + wr + i * 8 + (lane >> 2);
        const int cc = col0 + wc + j * 8 + 2 * (lane & 3) + h;
        if (r < m && cc < n) {
          const double v = alpha * acc[i][j][h];
          atomicAdd(C + (long)r * ldc + cc, v);
          if (sym && rt < ct) atomicAdd(C + (long)cc * ldc + r, v);
          if (trace && r == cc) atomicAdd(trace, v);
        }
      }
}

__global__ void __launch_bounds__(128) k_dgemm_split(bool ta, bool tb, bool sym, int m, int n, int k, int kslice,
                                                     double alpha, const double* __restrict__ A, int lda,
                                                     const double* __restrict__ B, int ldb, double* __restrict__ C,
                                                     int ldc) {
  if (sym && blockIdx.y > blockIdx.x) return;   // mirrored from tile (x, y)
  __shared__ SplitSmem sm;
  const int k0 = blockIdx.z * kslice, k1 = min(k, k0 + kslice);
  dgemm_tile(ta, tb, sym, m, n, blockIdx.y, blockIdx.x, k0, k1, alpha, A, lda, B, ldb, C, ldc, nullptr, sm);
}

// Small-matrix variant on warp units: one warp per (16 x 16 tile of C, 16-long
// k chunk), fragments of op(A) and op(B) loaded straight from global memory
// (L2-resident for these sizes), DMMA, then alpha * partial added to C with
// FP64 atomics (C pre-scaled by beta).  sym: only tiles on and above the
// diagonal, each added at its mirror as well.  With 16 DMMA per unit the work
// spreads evenly over every SM where 32 x 32 tiles leave SMs idle or doubled.
constexpr int WG_T = 16, WG_K = 16, WG_THREADS = 256;

__global__ void __launch_bounds__(WG_THREADS) k_dgemm_warp(bool ta, bool tb, bool sym, int m, int n, int k,
                                                           double alpha, const double* __restrict__ A, int lda,
                                                           const double* __restrict__ B, int ldb,
                                                           double* __restrict__ C, int ldc) {
  const int lane = threadIdx.x & 31;
  const int gwarp = blockIdx.x * (WG_THREADS / 32) + (threadIdx.x >> 5), nwarps = gridDim.x * (WG_THREADS / 32);
  const int mt = (m + WG_T - 1) / WG_T, ntl = (n + WG_T - 1) / WG_T, nkc = (k + WG_K - 1) / WG_K;
  const long ntiles = sym ? (long)ntl * (ntl + 1) / 2 : (long)mt * ntl;
  const long units = ntiles * nkc;
  const int r = lane >> 2, q = lane & 3;
  for (long u = gwarp; u < units; u += nwarps) {
    long t = u / nkc;
    const int kc = (int)(u - t * nkc);
    int rt, ct;
    if (sym) {
      rt = 0;
      while (t >= ntl - rt) {
        t -= ntl - rt;
        ++rt;
      }
      ct = rt + (int)t;
    } else {
      rt = (int)(t / ntl);
      ct = (int)(t - (long)rt * ntl);
    }
    const int k0 = kc * WG_K;
    double af[WG_K / 4][2], bf[WG_K / 4][2];
#pragma unroll
    for (int k4 = 0; k4 < WG_K / 4; ++k4) {
      const int kk = k0 + 4 * k4 + q;
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int row = rt * WG_T + 8 * i + r, col = ct * WG_T + 8 * i + r;
        double va = 0.0, vb = 0.0;
        if (row < m && kk < k) va = ta ? A[(long)kk * lda + row] : A[(long)row * lda + kk];
        if (col < n && kk < k) vb = tb ? B[(long)col * ldb + kk] : B[(long)kk * ldb + col];
        af[k4][i] = va;
        bf[k4][i] = vb;
      }
    }
    double acc[2][2][2] = {};
#pragma unroll
    for (int k4 = 0; k4 < WG_K / 4; ++k4)
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) dmma(acc[i][j][0], acc[i][j][1], af[k4][i], bf[k4][j]);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int row = rt * WG_T + 8 * i + r, col = ct * WG_T + 8 * j + 2 * q + h;
          if (row < m && col < n) {
            const double v = alpha * acc[i][j][h];
            atomicAdd(C + (long)row * ldc + col, v);
            if (sym && rt < ct) atomicAdd(C + (long)col * ldc + row, v);
          }
        }
  }
}

__global__ void k_scale_matrix(int m, int n, double beta, double* __restrict__ C, int ldc) {
  const int r = blockIdx.y, cc = blockIdx.x * blockDim.x + threadIdx.x;
  if (cc >= n) return;
  double* p = C + (long)r * ldc + cc;
  *p = beta == 0.0 ? 0.0 : beta * *p;
}

gbhf_status gemm(gbhf_ctx* c, bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda,
                 const double* B, int ldb, double beta, double* C, int ldc, bool sym) {
  if (m <= 0 || n <= 0) return GBHF_OK;
  sym = sym && m == n;
  const long tiles64 = (long)((n + GT - 1) / GT) * ((m + GT - 1) / GT);
  if (tiles64 >= 2L * c->nsm) {
    dim3 grid((n + GT - 1) / GT, (m + GT - 1) / GT);
    k_dgemm<<<grid, 128, 0, c->stream>>>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    count_launch(c);
    GBHF_CUDA(c, cudaGetLastError());
    return GBHF_OK;
  }
  if (m <= 1024 && n <= 1024) {
    // warp units: (16 x 16 tile, 16-long k chunk), about eight per SM or fewer
    const long t16 = sym ? (long)((n + WG_T - 1) / WG_T) * ((n + WG_T - 1) / WG_T + 1) / 2
                         : (long)((m + WG_T - 1) / WG_T) * ((n + WG_T - 1) / WG_T);
    const long units = t16 * ((k + WG_K - 1) / WG_K);
    const int grid = (int)std::max(1L, std::min<long>((units + WG_THREADS / 32 - 1) / (WG_THREADS / 32),
                                                      4L * c->nsm));
    k_scale_matrix<<<dim3((n + 127) / 128, m), 128, 0, c->stream>>>(m, n, beta, C, ldc);
    k_dgemm_warp<<<grid, WG_THREADS, 0, c->stream>>>(ta, tb, sym, m, n, k, alpha, A, lda, B, ldb, C, ldc);
    count_launch(c, 2);
    GBHF_CUDA(c, cudaGetLastError());
    return GBHF_OK;
  }
  const int nt = (n + ST - 1) / ST;
  const int tiles = sym ? nt * (nt + 1) / 2 : nt * ((m + ST - 1) / ST);
  int splits = std::max(1, (2 * c->nsm + tiles - 1) / tiles);
  splits = std::min(splits, std::max(1, (k + 4 * SK - 1) / (4 * SK)));   // at least 4 k-steps per slice
  int kslice = (k + splits - 1) / splits;
  kslice = (kslice + SK - 1) / SK * SK;
  splits = std::max(1, (k + kslice - 1) / kslice);
  k_scale_matrix<<<dim3((n + 127) / 128, m), 128, 0, c->stream>>>(m, n, beta, C, ldc);
  k_dgemm_split<<<dim3((n + ST - 1) / ST, (m + ST - 1) / ST, splits), 128, 0, c->stream>>>(
      ta, tb, sym, m, n, k, kslice, alpha, A, lda, B, ldb, C, ldc);
  count_launch(c, 2);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// ------------------------------------------------------- small kernels ----
__global__ void k_flat_to_square(int n, const double* __restrict__ f, double* __restrict__ s) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int a = min(i, j), b = max(i, j);
  s[(long)i * n + j] = f[(long)a * n - (long)a * (a - 1) / 2 + (b - a)];
}

__global__ void k_square_to_flat(int n, const double* __restrict__ s, double* __restrict__ f) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n || j < i) return;
  f[(long)i * n - (long)i * (i - 1) / 2 + (j - i)] = s[(long)i * n + j];
}

gbhf_status flat_to_square(gbhf_ctx* c, int n, const double* d_flat, double* d_sq) {
  k_flat_to_square<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, d_flat, d_sq);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

gbhf_status square_to_flat(gbhf_ctx* c, int n, const double* d_sq, double* d_flat) {
  k_square_to_flat<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, d_sq, d_flat);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

__global__ void k_axpby(size_t n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                        double* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = a * x[i] + (b == 0.0 ? 0.0 : b * y[i]);
}

gbhf_status axpby(gbhf_ctx* c, size_t n, double a, const double* x, double b, const double* y, double* out) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)c->nsm * 8);
  k_axpby<<<std::max(blocks, 1), 256, 0, c->stream>>>(n, a, x, b, y ? y : x, out);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// out = H + G + G^T (all square)
__global__ void k_add_sym(int n, const double* __restrict__ H, const double* __restrict__ G, double* __restrict__ out) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const long ij = (long)i * n + j, ji = (long)j * n + i;
  out[ij] = (H ? H[ij] : 0.0) + G[ij] + G[ji];
}

gbhf_status add_sym(gbhf_ctx* c, int n, const double* d_H, const double* d_Gpp, double* d_out) {
  k_add_sym<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, d_H, d_Gpp, d_out);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// e = M - M^T
__global__ void k_antisym(int n, const double* __restrict__ M, double* __restrict__ e) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  e[(long)i * n + j] = M[(long)i * n + j] - M[(long)j * n + i];
}

__global__ void k_to_float(size_t n, const double* __restrict__ x, float* __restrict__ y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

gbhf_status to_float(gbhf_ctx* c, size_t n, const double* d_x, float* d_y) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)c->nsm * 8);
  k_to_float<<<std::max(blocks, 1), 256, 0, c->stream>>>(n, d_x, d_y);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// Block reduction helper (sum or max) into a double.

// out[0] = max|e|, out[1] = 1/2 sum Dnew(H+F) (when H,F given), out[2] = sum (Dnew-Dold)^2,
// out[3] = sum(D (H + F)) with Dold (k_stats_grid below).
// Grid-wide reductions finish deterministically: each block reduces its slice
// and writes its partials, and the block that takes the last ticket combines
// the partials in block order (the same sums in the same order on every run)
// and returns the ticket to zero.
constexpr int RED_THREADS = 256, RED_MAXPART = 4096;

__device__ bool red_last_block(unsigned* ticket) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// k_stats over a grid: part[4 * block + q].
__global__ void __launch_bounds__(RED_THREADS) k_stats_grid(int n, const double* __restrict__ e,
    const double* __restrict__ H, const double* __restrict__ F, const double* __restrict__ Dn,
    const double* __restrict__ Do, double* __restrict__ part, unsigned* ticket, double* __restrict__ out) {
  double mx = 0, en = 0, dd = 0, eo = 0;
  const long nn = (long)n * n;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nn; i += (long)gridDim.x * blockDim.x) {
    if (e) mx = fmax(mx, fabs(e[i]));
    if (H && F && Dn) en += Dn[i] * (H[i] + F[i]);
    if (H && F && Do) eo += Do[i] * (H[i] + F[i]);
    if (Dn && Do) {
      const double d = Dn[i] - Do[i];
      dd += d * d;
    }
  }
  mx = block_reduce(mx, true);
  __syncthreads();
  en = block_reduce(en, false);
  __syncthreads();
  dd = block_reduce(dd, false);
  __syncthreads();
  eo = block_reduce(eo, false);
  if (threadIdx.x == 0) {
    part[4 * blockIdx.x + 0] = mx;
    part[4 * blockIdx.x + 1] = en;
    part[4 * blockIdx.x + 2] = dd;
    part[4 * blockIdx.x + 3] = eo;
  }
  if (red_last_block(ticket) && threadIdx.x == 0) {
    double m = 0, a = 0, b = 0, d = 0;
    for (unsigned g = 0; g < gridDim.x; ++g) {
      m = fmax(m, part[4 * g]);
      a += part[4 * g + 1];
      b += part[4 * g + 2];
      d += part[4 * g + 3];
    }
    out[0] = m;
    out[1] = 0.5 * a;
    out[2] = b;
    out[3] = 0.5 * d;
    *ticket = 0;
  }
}

static int red_blocks(gbhf_ctx* c, size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>((size_t)c->nsm, (n + 4 * RED_THREADS - 1) / (4 * RED_THREADS)));
}

static gbhf_status red_buffers(gbhf_ctx* c) {
  if (!c->red_ticket.p) {
    GBHF_CUDA(c, c->red_ticket.alloc(1));
    GBHF_CUDA(c, cudaMemsetAsync(c->red_ticket.p, 0, sizeof(unsigned), c->stream));
  }
  GBHF_CUDA(c, c->red_part.alloc(RED_MAXPART));
  return GBHF_OK;
}

gbhf_status reduce_stats(gbhf_ctx* c, int n, const double* d_e, const double* d_H, const double* d_F,
                         const double* d_Dnew, const double* d_Dold, double* host_out4) {
  GBHF_CUDA(c, c->small.alloc(64));
  GBHF_TRY(red_buffers(c));
  const int g = red_blocks(c, (size_t)n * n);
  k_stats_grid<<<g, RED_THREADS, 0, c->stream>>>(n, d_e, d_H, d_F, d_Dnew, d_Dold, c->red_part.p,
                                                c->red_ticket.p, c->small.p);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  // with a purification check pending, its record (small[12..14]) comes back in the same copy
  double h[PURIFY_REC + 3];
  const int nget = c->purify_pending ? PURIFY_REC + 3 : 4;
  GBHF_CUDA(c, cudaMemcpyAsync(h, c->small.p, nget * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  std::copy(h, h + 4, host_out4);
  if (c->purify_pending) GBHF_TRY(purify_finish(c, h + PURIFY_REC));
  return GBHF_OK;
}

__global__ void __launch_bounds__(RED_THREADS) k_max_abs(size_t n, const double* __restrict__ x,
                                                         double* __restrict__ part, unsigned* ticket, double* out) {
  double m = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(x[i]));
  m = block_reduce(m, true);
  if (threadIdx.x == 0) part[blockIdx.x] = m;
  if (red_last_block(ticket) && threadIdx.x == 0) {
    double r = 0;
    for (unsigned g = 0; g < gridDim.x; ++g) r = fmax(r, part[g]);
    *out = r;
    *ticket = 0;
  }
}

gbhf_status max_abs(gbhf_ctx* c, size_t n, const double* d_x, double* host_out) {
  GBHF_CUDA(c, c->small.alloc(64));
  GBHF_TRY(max_abs_dev(c, n, d_x, c->small.p + 8));
  GBHF_CUDA(c, cudaMemcpyAsync(host_out, c->small.p + 8, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

gbhf_status max_abs_dev(gbhf_ctx* c, size_t n, const double* d_x, double* d_out) {
  GBHF_TRY(red_buffers(c));
  k_max_abs<<<red_blocks(c, n), RED_THREADS, 0, c->stream>>>(n, d_x, c->red_part.p, c->red_ticket.p, d_out);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// out[j] = sum_i mats[j][i] * e[i], j < k  (DIIS B-matrix row; tr(e_j^T e) = sum e_j (.) e)
struct MatPtrs {
  const double* p[16];
};
// grid (G, k): block (g, j) sums slice g of mats[j] . e into part[j * G + g]
__global__ void __launch_bounds__(RED_THREADS) k_dots(size_t n2, int k, MatPtrs mats, const double* __restrict__ e,
                                                     double* __restrict__ part, unsigned* ticket,
                                                     double* __restrict__ out) {
  const int j = blockIdx.y, G = gridDim.x;
  const double* m = mats.p[j];
  double s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)G * blockDim.x) s += m[i] * e[i];
  s = block_reduce(s, false);
  if (threadIdx.x == 0) part[j * G + blockIdx.x] = s;
  if (red_last_block(ticket) && threadIdx.x == 0) {
    for (int jj = 0; jj < k; ++jj) {
      double t = 0;
      for (int g = 0; g < G; ++g) t += part[jj * G + g];
      out[jj] = t;
    }
    *ticket = 0;
  }
}

gbhf_status dot_matrices(gbhf_ctx* c, int n2, int k, const double* const* mats, const double* d_e, double* d_out) {
  if (k > 16) return fail(c, GBHF_ERR_BAD_INPUT, "too many DIIS vectors");
  MatPtrs mp;
  for (int j = 0; j < k; ++j) mp.p[j] = mats[j];
  GBHF_TRY(red_buffers(c));
  const int G = std::max(1, std::min(red_blocks(c, (size_t)n2), RED_MAXPART / 16));
  k_dots<<<dim3(G, k), RED_THREADS, 0, c->stream>>>((size_t)n2, k, mp, d_e, c->red_part.p, c->red_ticket.p, d_out);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// out = sum_j coefs[j] * mats[j]  (coefs in device memory)
__global__ void k_lincomb(size_t n2, int k, MatPtrs mats, const double* __restrict__ coefs, double* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) {
    double s = 0;
    for (int j = 0; j < k; ++j) s += coefs[j] * mats.p[j][i];
    out[i] = s;
  }
}

gbhf_status lincomb(gbhf_ctx* c, int n2, int k, const double* const* mats, const double* coefs, double* d_out) {
  if (k > 16) return fail(c, GBHF_ERR_BAD_INPUT, "too many DIIS vectors");
  MatPtrs mp;
  for (int j = 0; j < k; ++j) mp.p[j] = mats[j];
  int blocks = std::max(1, std::min((n2 + 255) / 256, c->nsm * 8));
  k_lincomb<<<blocks, 256, 0, c->stream>>>((size_t)n2, k, mp, coefs, d_out);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}


// Note: the reference evaluates alpha = mtx[i][k]/mtx[k][k] from the matrix
// before the pivot step for every j; updating j from m-1 down to k keeps
// a[i][k] unchanged until its own (last) update, which reproduces that.

__global__ void k_gauss(int m, const double* __restrict__ a_in, const double* __restrict__ b_in, double* __restrict__ x,
                        int* ok) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a[81], b[9];
  for (int i = 0; i < m * m; ++i) a[i] = a_in[i];
  for (int i = 0; i < m; ++i) b[i] = b_in[i];
  *ok = gauss_elem_dev(m, a, b, x) ? 1 : 0;
}

gbhf_status gauss_elem_dev_call(gbhf_ctx* c, int m, const double* h_a, const double* h_b, double* h_x, bool* ok) {
  if (m < 1 || m > 9) return fail(c, GBHF_ERR_BAD_INPUT, "gauss elimination: 1 <= m <= 9");
  GBHF_CUDA(c, c->small.alloc(256));
  double* da = c->small.p + 16;
  double* db = da + 81;
  double* dx = db + 9;
  int* dok = (int*)(dx + 9);
  GBHF_CUDA(c, cudaMemcpyAsync(da, h_a, m * m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(db, h_b, m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  k_gauss<<<1, 32, 0, c->stream>>>(m, da, db, dx, dok);
  count_launch(c);
  int hok = 0;
  GBHF_CUDA(c, cudaMemcpyAsync(h_x, dx, m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(&hok, dok, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  *ok = hok != 0;
  return GBHF_OK;
}

// --------------------------------------------------------------- Jacobi ----
// Parallel cyclic Jacobi (round-robin ordering) in one cooperative launch.
// The grid barrier spins with an iteration limit; on timeout it raises
// GBHF_DEV_ERR_TIMEOUT in *status and every block leaves.
constexpr long long BARRIER_SPIN_LIMIT = 1ll << 24;

// Every block adds one to *count and waits until it reaches epoch + gridDim.x
// (epoch counts the barriers passed times the grid size, the same in every
// block), so the last block to arrive releases the others with its own add; the
// counter starts at 0 with each launch.
__device__ bool grid_barrier(unsigned* count, unsigned& epoch, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  epoch += gridDim.x;
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(count, 1u);
    volatile unsigned* vc = count;
    long long it = 0;
    while (*vc < epoch) {
      if (++it > BARRIER_SPIN_LIMIT || *((volatile int*)status) & GBHF_DEV_ERR_TIMEOUT) {
        atomicOr(status, GBHF_DEV_ERR_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ void pair_of(int r, int k, int m, int& p, int& q) {
  // circle method: index m-1 fixed, others rotate
  if (k == 0) {
    p = r % (m - 1);
    q = m - 1;
  } else {
    p = (r + k) % (m - 1);
    q = (r - k + (m - 1)) % (m - 1);
  }
  if (p > q) {
    int t = p;
    p = q;
    q = t;
  }
}

// Rotation of the pair (p, q) that zeroes A_pq (Numerical Recipes form):
// c, s and t = s / c.  Every thread that needs it computes it from the same
// matrix, so all agree bit for bit.
__device__ __forceinline__ void jacobi_rot(const double* __restrict__ A, int m, int p, int q, double& c, double& s,
                                           double& t) {
  const double app = A[(long)p * m + p], aqq = A[(long)q * m + q], apq = A[(long)p * m + q];
  c = 1.0;
  s = 0.0;
  t = 0.0;
  if (apq != 0.0 && fabs(apq) > 1e-300 && !(fabs(apq) < 1e-18 * fmax(fabs(app), fabs(aqq)))) {
    const double theta = (aqq - app) / (2.0 * apq);
    if (fabs(theta) > 1e150) {
      t = 0.5 / theta;
    } else {
      t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
    }
    c = rsqrt(t * t + 1.0);
    s = t * c;
  }
}

// One grid barrier per round: the round reads A from one buffer and writes
// the rotated matrix to the other, each 2 x 2 block's thread computing the two
// rotations it needs from the unrotated matrix; V takes each round's rotations
// one round later from the parameters the diagonal blocks' threads stored.
__global__ void __launch_bounds__(256) k_jacobi(JacobiArgs a) {
  const int m = a.m, n = a.n, half = m / 2;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long gs = (long)gridDim.x * blockDim.x;
  unsigned* cnt = a.bar;
  unsigned epoch = 0;   // barrier target (grid_barrier)
  double* buf[2] = {a.A, a.A2};
  // Frobenius norm^2 of A (fixed under rotations)
  if (gt == 0) {
    a.red[0] = 0;
    a.red[1] = 0;
  }
  if (!grid_barrier(cnt, epoch, a.status)) return;
  {
    double s = 0;
    for (long i = gt; i < (long)m * m; i += gs) s += a.A[i] * a.A[i];
    s = block_reduce(s, false);
    if (threadIdx.x == 0) atomicAdd(&a.red[0], s);
  }
  if (!grid_barrier(cnt, epoch, a.status)) return;
  const double fro2 = a.red[0];
  const long nblk = (long)half * half;
  long g = 0;   // rounds done; round g reads buf[g & 1], writes buf[(g + 1) & 1]
  // V <- V J for the rotations of round gv (parameters in rot[(gv & 1) * 2m ..])
  auto apply_v = [&](long gv, long idx) {
    const int row = (int)(idx / half), P = (int)(idx % half);
    int p, q;
    pair_of((int)(gv % (m - 1)), P, m, p, q);
    const double* rt = a.rot + (gv & 1) * 2 * m;
    const double vp = a.V[(long)row * m + p], vq = a.V[(long)row * m + q];
    a.V[(long)row * m + p] = rt[2 * p] * vp + rt[2 * p + 1] * vq;
    a.V[(long)row * m + q] = rt[2 * q] * vq + rt[2 * q + 1] * vp;
  };
  int sweep = 0;
  for (; sweep < a.max_sweeps; ++sweep) {
    const double* Acur = buf[g & 1];
    // convergence test on the off-diagonal norm
    if (gt == 0) a.red[1] = 0;
    if (!grid_barrier(cnt, epoch, a.status)) return;
    {
      double s = 0;
      for (long i = gt; i < (long)m * m; i += gs) {
        const long r = i / m, cc = i % m;
        if (r != cc) s += Acur[i] * Acur[i];
      }
      s = block_reduce(s, false);
      if (threadIdx.x == 0) atomicAdd(&a.red[1], s);
    }
    if (!grid_barrier(cnt, epoch, a.status)) return;
    const double off2 = a.red[1];
    if (off2 <= a.tol * a.tol * fro2 || off2 == 0.0) break;
    for (int r = 0; r < m - 1; ++r, ++g) {
      const double* Ain = buf[g & 1];
      double* Aout = buf[(g + 1) & 1];
      double* rt = a.rot + (g & 1) * 2 * m;
      for (long idx = gt; idx < nblk + (g > 0 ? (long)n * half : 0); idx += gs) {
        if (idx >= nblk) {
          apply_v(g - 1, idx - nblk);   // the previous round's rotations
          continue;
        }
        const int P = (int)(idx / half), Qb = (int)(idx % half);
        if (Qb < P) continue;
        int p1, q1;
        pair_of(r, P, m, p1, q1);
        double c1, s1, t1;
        jacobi_rot(Ain, m, p1, q1, c1, s1, t1);
        if (P == Qb) {
          const double app = Ain[(long)p1 * m + p1], aqq = Ain[(long)q1 * m + q1], apq = Ain[(long)p1 * m + q1];
          Aout[(long)p1 * m + p1] = app - t1 * apq;
          Aout[(long)q1 * m + q1] = aqq + t1 * apq;
          const double off = t1 != 0.0 ? 0.0 : apq;
          Aout[(long)p1 * m + q1] = off;
          Aout[(long)q1 * m + p1] = off;
          rt[2 * p1] = c1;
          rt[2 * p1 + 1] = -s1;
          rt[2 * q1] = c1;
          rt[2 * q1 + 1] = s1;
        } else {
          int p2, q2;
          pair_of(r, Qb, m, p2, q2);
          double c2, s2, t2;
          jacobi_rot(Ain, m, p2, q2, c2, s2, t2);
          const int ii[2] = {p1, q1}, jj[2] = {p2, q2};
          const double ali[2] = {c1, c1}, bei[2] = {-s1, s1}, alj[2] = {c2, c2}, bej[2] = {-s2, s2};
          double old[2][2];
#pragma unroll
          for (int x = 0; x < 2; ++x)
#pragma unroll
            for (int y = 0; y < 2; ++y) old[x][y] = Ain[(long)ii[x] * m + jj[y]];
#pragma unroll
          for (int x = 0; x < 2; ++x)
#pragma unroll
            for (int y = 0; y < 2; ++y) {
              const double v = ali[x] * alj[y] * old[x][y] + ali[x] * bej[y] * old[x][1 - y] +
                               bei[x] * alj[y] * old[1 - x][y] + bei[x] * bej[y] * old[1 - x][1 - y];
              Aout[(long)ii[x] * m + jj[y]] = v;
              Aout[(long)jj[y] * m + ii[x]] = v;
            }
        }
      }
      if (!grid_barrier(cnt, epoch, a.status)) return;
    }
  }
  // the last round's rotations into V, and the final matrix into A
  if (g > 0)
    for (long idx = gt; idx < (long)n * half; idx += gs) apply_v(g - 1, idx);
  if (g & 1)
    for (long i = gt; i < (long)m * m; i += gs) a.A[i] = a.A2[i];
  if (gt == 0) {
    *a.sweeps_out = sweep;
    if (sweep >= a.max_sweeps) atomicOr(a.status, GBHF_DEV_ERR_NOTCONV);
  }
}

// ascending sort of the diagonal with the matching columns
__global__ void k_sort_eig(int n, int m, const double* __restrict__ A, const double* __restrict__ V,
                           double* __restrict__ evals, double* __restrict__ evecs) {
  // one block; rank by (value, index)
  __shared__ double sv[1024];
  __shared__ int rank[1024];
  for (int i = threadIdx.x; i < n; i += blockDim.x) sv[i] = A[(long)i * m + i];
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int r = 0;
    const double vi = sv[i];
    for (int j = 0; j < n; ++j) {
      const double vj = sv[j];
      if (vj < vi || (vj == vi && j < i)) ++r;
    }
    rank[i] = r;
    evals[r] = vi;
  }
  __syncthreads();
  for (long idx = threadIdx.x; idx < (long)n * n; idx += blockDim.x) {
    const int row = (int)(idx / n), col = (int)(idx % n);
    evecs[(long)row * n + rank[col]] = V[(long)row * m + col];
  }
}

__global__ void k_jacobi_init(int n, int m, const double* __restrict__ Ain, double* __restrict__ A,
                              double* __restrict__ V) {
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < (long)m * m; idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / m), j = (int)(idx % m);
    A[idx] = (i < n && j < n) ? Ain[(long)i * n + j] : 0.0;
    if (i < n) V[(long)i * m + j] = (i == j) ? 1.0 : 0.0;
  }
}

// d_evecs (n x n): eigenvectors of A in columns, ascending eigenvalues.
// Up to TRIDIAG_MAX_N: Householder tridiagonalisation, bisection and inverse
// iteration (tridiag.cu; the warm start d_V0 is not needed there).  Above it,
// or with GBHF_EIGEN=jacobi: the Jacobi solver below.
gbhf_status eigh(gbhf_ctx* c, int n, const double* d_A, double* d_evals, double* d_evecs, const double* d_V0) {
  if (n <= 0 || n > 1024) return fail(c, GBHF_ERR_UNSUPPORTED, "eigen-solve supports 1 <= n <= 1024");
  if (n <= TRIDIAG_MAX_N && !c->force_jacobi && tridiag_smem_bytes(n) <= c->smem_optin)
    return eigh_tridiag(c, n, d_A, d_evals, d_evecs);
  JacobiWork& w = c->jac;
  const int mm = std::max(2, n + (n & 1));
  GBHF_CUDA(c, w.A.alloc((size_t)mm * mm));
  GBHF_CUDA(c, w.A2.alloc((size_t)mm * mm));
  GBHF_CUDA(c, w.V.alloc((size_t)n * mm));
  GBHF_CUDA(c, w.rot.alloc(4 * (size_t)mm));
  GBHF_CUDA(c, w.red.alloc(4));
  GBHF_CUDA(c, w.sweeps.alloc(1));
  GBHF_CUDA(c, w.bar.alloc(2));
  GBHF_CUDA(c, c->dev_status.alloc(1));
  GBHF_CUDA(c, cudaMemsetAsync(w.bar.p, 0, 2 * sizeof(unsigned), c->stream));
  GBHF_CUDA(c, cudaMemsetAsync(c->dev_status.p, 0, sizeof(int), c->stream));
  // optional warm start: A' = V0^T A V0 (V0 orthogonal), eigenvectors = V0 * W
  const double* src = d_A;
  GBHF_CUDA(c, w.t1.alloc((size_t)n * n));
  GBHF_CUDA(c, w.t2.alloc((size_t)n * n));
  GBHF_CUDA(c, w.t3.alloc((size_t)n * n));
  if (d_V0) {
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, d_A, n, d_V0, n, 0.0, w.t1.p, n));
    GBHF_TRY(gemm(c, true, false, n, n, n, 1.0, d_V0, n, w.t1.p, n, 0.0, w.t2.p, n));
    src = w.t2.p;
  }
  k_jacobi_init<<<std::max(1, std::min(c->nsm * 4, (mm * mm + 255) / 256)), 256, 0, c->stream>>>(n, mm, src, w.A.p,
                                                                                                   w.V.p);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_jacobi_init launch");
  JacobiArgs a;
  a.n = n;
  a.m = mm;
  a.A = w.A.p;
  a.A2 = w.A2.p;
  a.V = w.V.p;
  a.rot = w.rot.p;
  a.red = w.red.p;
  a.bar = w.bar.p;
  a.status = c->dev_status.p;
  a.max_sweeps = 40;
  a.tol = 1e-14;
  a.sweeps_out = w.sweeps.p;
  if (w.grid == 0) {
    int per_sm = 0;
    GBHF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi, 256, 0));
    w.grid = std::max(1, c->nsm * std::min(per_sm, 2));
  }
  const long work = (long)(mm / 2) * (mm / 2) + (long)n * (mm / 2);
  const int grid = (int)std::max(1L, std::min<long>(w.grid, (work + 255) / 256));
  void* args[] = {&a};
  GBHF_CUDA(c, cudaLaunchCooperativeKernel((void*)k_jacobi, dim3(grid), dim3(256), args, 0, c->stream));
  count_launch(c);
  double* vec_out = d_V0 ? w.t3.p : d_evecs;
  k_sort_eig<<<1, 1024, 0, c->stream>>>(n, mm, w.A.p, w.V.p, d_evals, vec_out);
  count_launch(c);
  GBHF_LAUNCHED(c, "k_sort_eig launch");
  if (d_V0) GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, d_V0, n, w.t3.p, n, 0.0, d_evecs, n));
  int st = 0, sweeps = 0;
  GBHF_CUDA(c, cudaMemcpyAsync(&st, c->dev_status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(&sweeps, w.sweeps.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  GBHF_CUDA(c, cudaGetLastError());
  w.last_sweeps = sweeps;
  c->prof.jacobi_sweeps += sweeps;
  c->prof.jacobi_calls += 1;
  if (st & GBHF_DEV_ERR_TIMEOUT) return fail(c, GBHF_ERR_DEVICE_TIMEOUT, "Jacobi grid barrier timed out");
  if (st & GBHF_DEV_ERR_NOTCONV) return fail(c, GBHF_ERR_NOT_CONVERGED, "Jacobi eigen-solver did not converge");
  return GBHF_OK;
}

// --------------------------------------------- GEMM-only matrix functions ----
// Gershgorin interval and trace of a symmetric matrix: out = {lo, hi, trace}.
__global__ void k_gershgorin(int n, const double* __restrict__ A, double* __restrict__ out) {
  // a warp per row (coalesced loads), the warps of the block taking rows in turn
  double lo = 1e300, hi = -1e300, tr = 0;
  {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wid; i < n; i += nw) {
      const double* row = A + (long)i * n;
      double r = 0;
      for (int j = lane; j < n; j += 32)
        if (j != i) r += fabs(row[j]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
      const double d = row[i];
      lo = fmin(lo, d - r);
      hi = fmax(hi, d + r);
      if (lane == 0) tr += d;
    }
  }
  __shared__ double s_lo[32], s_hi[32], s_tr[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    tr += __shfl_xor_sync(0xffffffffu, tr, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    s_lo[wid] = lo;
    s_hi[wid] = hi;
    s_tr[wid] = tr;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; ++w) {
      lo = fmin(lo, s_lo[w]);
      hi = fmax(hi, s_hi[w]);
      tr += s_tr[w];
    }
    out[0] = lo;
    out[1] = hi;
    out[2] = tr;
  }
}

// P0 = (lambda/n)(mu I - F) + (ne/n) I with mu = tr F / n and
// lambda = min(ne/(hi - mu), (n - ne)/(mu - lo))  (canonical purification start).
__global__ void k_purify_init(int n, int ne, const double* __restrict__ F, const double* __restrict__ g,
                              double* __restrict__ P) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double lo = g[0], hi = g[1], mu = g[2] / n;
  double lam = 1e300;
  if (hi - mu > 0) lam = fmin(lam, ne / (hi - mu));
  if (mu - lo > 0) lam = fmin(lam, (n - ne) / (mu - lo));
  if (!(lam < 1e300)) lam = 0;
  const double f = F[(long)i * n + j];
  P[(long)i * n + j] = (lam / n) * ((i == j ? mu : 0.0) - f) + (i == j ? (double)ne / n : 0.0);
}

// traces of P, P^2, P^3 (diagonals) -> coefficients of the next iterate
// P' = a P + b P^2 + d P^3 and the idempotency error tr(P - P^2) in coef[3].
__global__ void k_purify_coef(int n, const double* __restrict__ P, const double* __restrict__ P2,
                              const double* __restrict__ P3, double* __restrict__ coef) {
  double t1 = 0, t2 = 0, t3 = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    t1 += P[(long)i * n + i];
    t2 += P2[(long)i * n + i];
    t3 += P3[(long)i * n + i];
  }
  __shared__ double s[3][32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t1 += __shfl_xor_sync(0xffffffffu, t1, o);
    t2 += __shfl_xor_sync(0xffffffffu, t2, o);
    t3 += __shfl_xor_sync(0xffffffffu, t3, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    s[0][wid] = t1;
    s[1][wid] = t2;
    s[2][wid] = t3;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; ++w) {
      t1 += s[0][w];
      t2 += s[1][w];
      t3 += s[2][w];
    }
    const double den = t1 - t2, num = t2 - t3;
    double a, b, d;
    if (!(fabs(den) > 1e-300)) {   // already idempotent: keep P
      a = 1;
      b = 0;
      d = 0;
    } else {
      const double cc = num / den;
      if (cc >= 0.5) {
        a = 0;
        b = (1 + cc) / cc;
        d = -1 / cc;
      } else {
        a = (1 - 2 * cc) / (1 - cc);
        b = (1 + cc) / (1 - cc);
        d = -1 / (1 - cc);
      }
    }
    coef[0] = a;
    coef[1] = b;
    coef[2] = d;
    coef[3] = den;
  }
}

// The canonical purification (two GEMMs per step) in one cooperative launch;
// the trace-correcting one runs in k_tc2_fused below.  Per step the symmetric
// products P2 = P P and P3 = P P2 are shared out as (upper tile, k slice) items
// with atomic accumulation, their traces summed in the tile epilogues; then
// every block derives the step's coefficients from the same three traces (so
// all blocks take the same decision to stop) and updates its share of P while
// clearing P2 and P3 for the next step.  Three bounded grid barriers per step.
// Trace slots tr[3 * parity + {0, 1, 2}] (tr P, tr P2, tr P3) alternate between
// steps; P2, P3 and tr must be zero at launch.
struct PurifyArgs {
  int n, ne, nt, ks, kslice, max_steps;
  int tc2;                          // 1: trace-correcting steps (one GEMM per step), 0: canonical
  double tol;
  double *P, *P2, *P3, *tr, *out;   // out: [0] last tr(P - P^2), [1] steps
  unsigned* bar;
  int* status;
};

__global__ void __launch_bounds__(128) k_purify_fused(PurifyArgs a) {
  __shared__ SplitSmem sm;
  __shared__ double s_red[4];
  const int n = a.n;
  const long nn = (long)n * n;
  const int ntile = a.nt * (a.nt + 1) / 2, items = ntile * a.ks;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x, gs = (long)gridDim.x * blockDim.x;
  unsigned* cnt = a.bar;
  unsigned epoch = 0;   // barrier target (grid_barrier)
  auto block_sum_add = [&](double v, double* dst) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      const double t = s_red[0] + s_red[1] + s_red[2] + s_red[3];
      if (t != 0.0) atomicAdd(dst, t);
    }
    __syncthreads();
  };
  // upper-triangle tile index -> (row tile, column tile)
  auto tile_of = [&](int t, int& rt, int& ct) {
    rt = 0;
    while (t >= a.nt - rt) {
      t -= a.nt - rt;
      ++rt;
    }
    ct = rt + t;
  };
  {
    double v = 0;
    for (long i = gt; i < n; i += gs) v += a.P[i * n + i];
    block_sum_add(v, a.tr);
  }
  if (!grid_barrier(cnt, epoch, a.status)) return;
  int step = 0;
  for (; step < a.max_steps; ++step) {
    double* trp = a.tr + 3 * (step & 1);
    double* trq = a.tr + 3 * ((step + 1) & 1);
    if (gt == 0) {   // the other parity: read last in the previous step's coefficients
      trq[0] = 0.0;
      trq[1] = 0.0;
      trq[2] = 0.0;
    }
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
      int rt, ct;
      tile_of(it / a.ks, rt, ct);
      const int k0 = (it % a.ks) * a.kslice, k1 = min(n, k0 + a.kslice);
      dgemm_tile(false, false, true, n, n, rt, ct, k0, k1, 1.0, a.P, n, a.P, n, a.P2, n, trp + 1, sm);
    }
    if (!grid_barrier(cnt, epoch, a.status)) return;
    if (a.tc2) {
      // trace-correcting step: P <- P^2 or 2P - P^2, whichever brings tr toward ne
      const double t1 = *((volatile double*)trp), t2 = *((volatile double*)(trp + 1));
      const double den = t1 - t2;
      if (gt == 0) {
        a.out[0] = den;
        a.out[1] = step + 1;
      }
      if (fabs(den) < a.tol * max(1, a.ne)) break;   // the same decision in every block
      const bool sq = fabs(t2 - a.ne) < fabs(2 * t1 - t2 - a.ne);
      const double ca = sq ? 0.0 : 2.0, cb = sq ? 1.0 : -1.0;
      double dsum = 0;
      for (long e = gt; e < nn; e += gs) {
        const double v = ca * a.P[e] + cb * a.P2[e];
        a.P[e] = v;
        a.P2[e] = 0.0;
        if (e / n == e % n) dsum += v;
      }
      block_sum_add(dsum, trq);
      if (!grid_barrier(cnt, epoch, a.status)) return;
      continue;
    }
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
      int rt, ct;
      tile_of(it / a.ks, rt, ct);
      const int k0 = (it % a.ks) * a.kslice, k1 = min(n, k0 + a.kslice);
      dgemm_tile(false, false, true, n, n, rt, ct, k0, k1, 1.0, a.P, n, a.P2, n, a.P3, n, trp + 2, sm);
    }
    if (!grid_barrier(cnt, epoch, a.status)) return;
    const double t1 = *((volatile double*)trp), t2 = *((volatile double*)(trp + 1)),
                 t3 = *((volatile double*)(trp + 2));
    const double den = t1 - t2, num = t2 - t3;
    if (gt == 0) {
      a.out[0] = den;
      a.out[1] = step + 1;
    }
    if (fabs(den) < a.tol * max(1, a.ne)) break;   // the same decision in every block
    double ca = 1, cb = 0, cd = 0;
    if (fabs(den) > 1e-300) {
      const double cc = num / den;
      if (cc >= 0.5) {
        ca = 0;
        cb = (1 + cc) / cc;
        cd = -1 / cc;
      } else {
        ca = (1 - 2 * cc) / (1 - cc);
        cb = (1 + cc) / (1 - cc);
        cd = -1 / (1 - cc);
      }
    }
    double dsum = 0;
    for (long e = gt; e < nn; e += gs) {
      const double v = ca * a.P[e] + cb * a.P2[e] + cd * a.P3[e];
      a.P[e] = v;
      a.P2[e] = 0.0;
      a.P3[e] = 0.0;
      if (e / n == e % n) dsum += v;
    }
    block_sum_add(dsum, trq);
    if (!grid_barrier(cnt, epoch, a.status)) return;
  }
}

// Trace-correcting purification with one grid barrier per step.  Step s
// computes P2_s = P_s P_s while P_s itself is only formed on the fly:
// P_s = ca P_(s-1) + cb P2_(s-1) (tc2_next) when the GEMM tiles are loaded, and
// written out (for step s + 1) by a strided pass that runs beside the GEMM.
// P alternates between two buffers, P2 rotates over three (the one zeroed in
// step s was last read in step s - 1), and the traces of P_s and P2_s sit in
// three rotating slots, so that the single barrier at the end of a step is the
// only ordering needed.  After the barrier every block takes the same step
// decision from the same two traces.
struct Tc2Args {
  int n, ne, max_steps;
  double tol;
  double *P0, *P1;        // P0 holds P_0 at launch; the result is copied back there
  double *Q0, *Q1, *Q2;   // the three P2 buffers, zero at launch
  double* tr;        // 6 slots: tr P_s at 2 (s % 3), tr P2_s at 2 (s % 3) + 1; zero at launch
  double* out;       // [0] last tr(P - P^2), [1] steps
  unsigned* bar;
  int* status;
};

// The one formula for an element of P_s, used by the GEMM loads and by the
// pass that writes P_s out, so that both give the same bits.
__device__ __forceinline__ double tc2_next(double ca, double cb, double p, double p2) {
  return __fma_rn(ca, p, __dmul_rn(cb, p2));
}

// GEMM units of a step: (16 x 16 tile on or above the diagonal, 16-long k
// chunk), one warp each, fragments loaded straight from global memory (P_s is
// exactly symmetric, so the column fragment of B is a row fragment of P_s) and
// multiplied by DMMA; the tile (and its mirror) is added into P2_s with FP64
// atomics.  256 threads per block.
constexpr int TC2_THREADS = 256, TC2_T = 16, TC2_K = 16;

__global__ void __launch_bounds__(TC2_THREADS) k_tc2_fused(Tc2Args a) {
  __shared__ double s_red[TC2_THREADS / 32];
  const int n = a.n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long nn = (long)n * n;
  const int nt = (n + TC2_T - 1) / TC2_T, nkc = (n + TC2_K - 1) / TC2_K;
  const int units = nt * (nt + 1) / 2 * nkc;
  const int gwarp = blockIdx.x * (TC2_THREADS / 32) + warp, nwarps = gridDim.x * (TC2_THREADS / 32);
  const long gt = blockIdx.x * (long)blockDim.x + tid, gs = (long)gridDim.x * blockDim.x;
  unsigned epoch = 0;
  auto block_sum_add = [&](double v, double* dst) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
#pragma unroll
      for (int w = 0; w < TC2_THREADS / 32; ++w) t += s_red[w];
      if (t != 0.0) atomicAdd(dst, t);
    }
    __syncthreads();
  };
  auto pbuf = [&](int i) -> double* { return i == 0 ? a.P0 : a.P1; };
  auto qbuf = [&](int i) -> double* { return i == 0 ? a.Q0 : (i == 1 ? a.Q1 : a.Q2); };
  {
    double v = 0;
    for (long i = gt; i < n; i += gs) v += a.P0[i * n + i];
    block_sum_add(v, a.tr);   // tr P_0 in slot 0
  }
  if (!grid_barrier(a.bar, epoch, a.status)) return;
  double ca = 1.0, cb = 0.0;   // P_s = ca P_(s-1) + cb P2_(s-1); step 0 reads P_0 as it is
  int step = 0, final_buf = 0;
  for (; step < a.max_steps; ++step) {
    const double* Pin = pbuf(step == 0 ? 0 : (step - 1) & 1);   // P_(s-1) (P_0 at step 0)
    const double* P2in = qbuf(step == 0 ? 2 : (step - 1) % 3);  // P2_(s-1) (zero at step 0)
    double* Pout = pbuf(step & 1);
    double* P2out = qbuf(step % 3);
    double* trp = a.tr + 2 * (step % 3);
    // the slots of step s + 1, last read after the barrier of step s - 2
    if (gt == 0) {
      a.tr[2 * ((step + 1) % 3)] = 0.0;
      a.tr[2 * ((step + 1) % 3) + 1] = 0.0;
    }
    if (step > 0) {
      // P_s written out with its trace (step 0: P_0 is already in P0), and the
      // P2 buffer of step s + 1 cleared (it held P2_(s-2), read during step s - 1)
      double* z = qbuf((step + 1) % 3);
      double dsum = 0;
      for (long e = gt; e < nn; e += gs) {
        const double v = tc2_next(ca, cb, Pin[e], P2in[e]);
        Pout[e] = v;
        z[e] = 0.0;
        if (e / n == e % n) dsum += v;
      }
      block_sum_add(dsum, trp);
    }
    // P2_s = P_s P_s
    double dtr = 0.0;
    for (int u = gwarp; u < units; u += nwarps) {
      int t = u / nkc;
      const int kc = u - t * nkc;
      int rt = 0;
      while (t >= nt - rt) {
        t -= nt - rt;
        ++rt;
      }
      const int ct = rt + t;
      const int k0 = kc * TC2_K;
      const int r = lane >> 2, q = lane & 3;
      double af[TC2_K / 4][2], bf[TC2_K / 4][2];
#pragma unroll
      for (int k4 = 0; k4 < TC2_K / 4; ++k4) {
        const int k = k0 + 4 * k4 + q;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int row = rt * TC2_T + 8 * i + r, col = ct * TC2_T + 8 * i + r;
          double va = 0.0, vb = 0.0;
          if (row < n && k < n) va = tc2_next(ca, cb, Pin[(long)row * n + k], P2in[(long)row * n + k]);
          if (col < n && k < n) vb = tc2_next(ca, cb, Pin[(long)col * n + k], P2in[(long)col * n + k]);
          af[k4][i] = va;
          bf[k4][i] = vb;
        }
      }
      double acc[2][2][2] = {};
#pragma unroll
      for (int k4 = 0; k4 < TC2_K / 4; ++k4)
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j) dmma(acc[i][j][0], acc[i][j][1], af[k4][i], bf[k4][j]);
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int row = rt * TC2_T + 8 * i + r, col = ct * TC2_T + 8 * j + 2 * q + h;
            if (row < n && col < n) {
              const double v = acc[i][j][h];
              atomicAdd(P2out + (long)row * n + col, v);
              if (rt < ct) atomicAdd(P2out + (long)col * n + row, v);
              if (row == col) dtr += v;
            }
          }
    }
    block_sum_add(dtr, trp + 1);
    if (!grid_barrier(a.bar, epoch, a.status)) return;
    // the same decision in every block
    const double t1 = *((volatile double*)trp), t2 = *((volatile double*)(trp + 1));
    const double den = t1 - t2;
    if (gt == 0) {
      a.out[0] = den;
      a.out[1] = step + 1;
    }
    final_buf = step == 0 ? 0 : (step & 1);
    if (fabs(den) < a.tol * max(1, a.ne)) break;
    const bool sq = fabs(t2 - a.ne) < fabs(2 * t1 - t2 - a.ne);
    ca = sq ? 0.0 : 2.0;
    cb = sq ? 1.0 : -1.0;
  }
  // the converged P_s back into P0
  if (final_buf != 0)
    for (long e = gt; e < nn; e += gs) a.P0[e] = a.P1[e];
}

// TC2 start: the spectrum of F mapped onto [0, 1], reversed (P0 = (hi I - F) / (hi - lo)).
__global__ void k_tc2_init(int n, const double* __restrict__ F, const double* __restrict__ g, double* __restrict__ P,
                           double* __restrict__ Q0, double* __restrict__ Q1, double* __restrict__ Q2,
                           double* __restrict__ tr, unsigned* __restrict__ bar, int* __restrict__ status) {
  // P0 = (hi I - F) / (hi - lo), and the zeros the fused kernel starts from
  // (its three P^2 buffers, trace slots, barrier counter and status word)
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && blockIdx.x == 0) {
    if (threadIdx.x < 16) tr[threadIdx.x] = 0.0;
    if (threadIdx.x < 2) bar[threadIdx.x] = 0u;
    if (threadIdx.x == 0) *status = 0;
  }
  if (j >= n) return;
  const double lo = g[0], hi = g[1];
  const double sc = hi > lo ? 1.0 / (hi - lo) : 0.0;
  const long e = (long)i * n + j;
  P[e] = sc * ((i == j ? hi : 0.0) - F[e]);
  Q0[e] = 0.0;
  Q1[e] = 0.0;
  Q2[e] = 0.0;
}

// The spectral projector onto the ne lowest eigenvectors of the symmetric F.
// Trace-correcting purification (TC2; Niklasson, Phys. Rev. B 66, 155115 (2002)):
// P <- P^2 or 2P - P^2 by the trace, one GEMM per step; on water clusters it
// needs ~24 steps where the canonical purification (Palser & Manolopoulos,
// Phys. Rev. B 58, 12704 (1998); trace-conserving cubic polynomials, two GEMMs
// per step, tc2 = false) needs ~17, so a third fewer GEMMs.  TC2 runs the
// one-barrier kernel k_tc2_fused.  Returns the idempotency error tr(P - P^2)
// of the result.
// The purification record (final error, steps, device status) for a deferred check.
__global__ void k_purify_record(const double* __restrict__ out, const int* __restrict__ st, double* __restrict__ rec) {
  rec[0] = out[0];
  rec[1] = out[1];
  rec[2] = (double)*st;
}

gbhf_status purify(gbhf_ctx* c, int n, int ne, const double* d_F, double* d_P, double* err_out, bool tc2) {
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, P2, 23, nn);
  GBHF_CUDA(c, c->jac.t1.alloc(nn));
  double* P3 = c->jac.t1.p;
  GBHF_CUDA(c, c->small.alloc(64));
  double* g = c->small.p + 32;
  double* tr = c->small.p + 40;   // 6 trace slots
  double* out = c->small.p + 48;
  GBHF_CUDA(c, c->jac.bar.alloc(2));
  GBHF_CUDA(c, c->dev_status.alloc(1));
  k_gershgorin<<<1, 1024, 0, c->stream>>>(n, d_F, g);
  count_launch(c);
  if (tc2) {
    GBHF_CUDA(c, c->jac.t2.alloc(nn));
    GBHF_CUDA(c, c->jac.t3.alloc(nn));
    k_tc2_init<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, d_F, g, d_P, P2, P3, c->jac.t2.p, tr,
                                                                c->jac.bar.p, c->dev_status.p);
    count_launch(c);
  } else {
    k_purify_init<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, ne, d_F, g, d_P);
    count_launch(c);
    GBHF_CUDA(c, cudaMemsetAsync(P2, 0, nn * sizeof(double), c->stream));
    GBHF_CUDA(c, cudaMemsetAsync(P3, 0, nn * sizeof(double), c->stream));
    GBHF_CUDA(c, cudaMemsetAsync(tr, 0, 16 * sizeof(double), c->stream));
    GBHF_CUDA(c, cudaMemsetAsync(c->jac.bar.p, 0, 2 * sizeof(unsigned), c->stream));
    GBHF_CUDA(c, cudaMemsetAsync(c->dev_status.p, 0, sizeof(int), c->stream));
  }
  const int nt = (n + ST - 1) / ST;
  const int ntile = nt * (nt + 1) / 2;
  // k slices: about one item per SM, at least two k-steps per slice
  const int ks0 = std::max(1, std::min((c->nsm + ntile - 1) / ntile, (n + 2 * SK - 1) / (2 * SK)));
  const int kslice = ((n + ks0 - 1) / ks0 + SK - 1) / SK * SK;
  const int ks = (n + kslice - 1) / kslice;
  double hout[2] = {1.0, 0.0};
  if (tc2) {
    // one barrier per step: a second P buffer and three P2 buffers (zeroed by k_tc2_init)
    Tc2Args t;
    t.n = n;
    t.ne = ne;
    t.max_steps = 200;
    t.tol = 1e-13;   // E[D] is first order in the idempotency error
    t.P0 = d_P;
    t.P1 = c->jac.t3.p;
    t.Q0 = P2;
    t.Q1 = P3;
    t.Q2 = c->jac.t2.p;
    t.tr = tr;
    t.out = out;
    t.bar = c->jac.bar.p;
    t.status = c->dev_status.p;
    if (c->tc2_grid == 0) {
      int per_sm = 0;
      GBHF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tc2_fused, TC2_THREADS, 0));
      c->tc2_grid = std::max(1, c->nsm * std::min(std::max(per_sm, 1), 2));
    }
    const int nt16 = (n + TC2_T - 1) / TC2_T;
    const long units = (long)nt16 * (nt16 + 1) / 2 * ((n + TC2_K - 1) / TC2_K);
    const int grid = (int)std::max(1L, std::min<long>(c->tc2_grid, (units + 7) / 8));
    void* args[] = {&t};
    GBHF_CUDA(c, cudaLaunchCooperativeKernel((void*)k_tc2_fused, dim3(grid), dim3(TC2_THREADS), args, 0, c->stream));
    count_launch(c);
  } else {
    PurifyArgs a;
    a.n = n;
    a.ne = ne;
    a.nt = nt;
    a.kslice = kslice;
    a.ks = ks;
    a.max_steps = 200;
    a.tc2 = tc2 ? 1 : 0;
    a.tol = 1e-13;   // E[D] is first order in the idempotency error
    a.P = d_P;
    a.P2 = P2;
    a.P3 = P3;
    a.tr = tr;
    a.out = out;
    a.bar = c->jac.bar.p;
    a.status = c->dev_status.p;
    if (c->purify_grid == 0) {
      int per_sm = 0;
      GBHF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_purify_fused, 128, 0));
      c->purify_grid = std::max(1, c->nsm * std::max(per_sm, 1));
    }
    const int grid = std::max(1, std::min(c->purify_grid, ntile * a.ks));
    void* args[] = {&a};
    GBHF_CUDA(c, cudaLaunchCooperativeKernel((void*)k_purify_fused, dim3(grid), dim3(128), args, 0, c->stream));
    count_launch(c);
  }
  c->purify_ne = ne;
  if (c->purify_defer && !err_out) {
    // the record (error, steps, device status) waits in small[16..18] for the
    // caller's next read (reduce_stats), which runs purify_finish
    GBHF_CUDA(c, c->small.alloc(64));
    k_purify_record<<<1, 1, 0, c->stream>>>(out, c->dev_status.p, c->small.p + PURIFY_REC);
    count_launch(c);
    GBHF_CUDA(c, cudaGetLastError());
    c->purify_pending = true;
    return GBHF_OK;
  }
  int st = 0;
  GBHF_CUDA(c, cudaMemcpyAsync(hout, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(&st, c->dev_status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  const double rec[3] = {hout[0], hout[1], (double)st};
  if (err_out) *err_out = hout[0];
  c->purify_pending = true;
  return purify_finish(c, rec);
}

gbhf_status purify_flush(gbhf_ctx* c) {
  if (!c->purify_pending) return GBHF_OK;
  double rec[3];
  GBHF_CUDA(c, cudaMemcpyAsync(rec, c->small.p + PURIFY_REC, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return purify_finish(c, rec);
}

gbhf_status purify_finish(gbhf_ctx* c, const double* rec) {
  c->purify_pending = false;
  const int st = (int)rec[2];
  if (st & GBHF_DEV_ERR_TIMEOUT) return fail(c, GBHF_ERR_DEVICE_TIMEOUT, "purification grid barrier timed out");
  c->prof.purify_steps += rec[1];
  c->prof.purify_calls += 1;
  if (!(std::fabs(rec[0]) < 1e-6 * std::max(1, c->purify_ne)))
    return fail(c, GBHF_ERR_NOT_CONVERGED, "density purification did not converge");
  return GBHF_OK;
}

// Density of the ne lowest orbitals of F (AO basis) in the orthogonalised
// basis: D = X (2 P) X^T with P the projector of F' = X^T F X.
gbhf_status density_purified_dev(gbhf_ctx* c, int n, const double* d_Fsq, const double* d_X, int nocc,
                                 double* d_Dsq) {
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, T1, 10, nn);
  GBHF_WS(c, Fp, 11, nn);
  GBHF_WS(c, P, 12, nn);
  GBHF_TRY(gemm(c, true, false, n, n, n, 1.0, d_X, n, d_Fsq, n, 0.0, T1, n));
  GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, T1, n, d_X, n, 0.0, Fp, n, true));
  if (nocc <= 0) {
    GBHF_CUDA(c, cudaMemsetAsync(d_Dsq, 0, nn * sizeof(double), c->stream));
    return GBHF_OK;
  }
  GBHF_TRY(purify(c, n, nocc, Fp, P, nullptr));
  GBHF_TRY(gemm(c, false, false, n, n, n, 2.0, d_X, n, P, n, 0.0, T1, n));
  GBHF_TRY(gemm(c, false, true, n, n, n, 1.0, T1, n, d_X, n, 0.0, d_Dsq, n, true));
  return GBHF_OK;
}

// 3I - M
__global__ void k_three_minus(int n, const double* __restrict__ M, double* __restrict__ out) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  out[(long)i * n + j] = (i == j ? 3.0 : 0.0) - M[(long)i * n + j];
}

__global__ void k_ns_init(int n, const double* __restrict__ S, const double* __restrict__ g, double* __restrict__ Y,
                          double* __restrict__ Z) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double scale = 1.0 / g[1];
  Y[(long)i * n + j] = S[(long)i * n + j] * scale;
  Z[(long)i * n + j] = i == j ? 1.0 : 0.0;
}

__global__ void k_ns_err(int n, const double* __restrict__ T, double* out) {
  double m = 0;
  for (long idx = threadIdx.x; idx < (long)n * n; idx += blockDim.x) {
    const long i = idx / n, j = idx % n;
    m = fmax(m, fabs(T[idx] - (i == j ? 1.0 : 0.0)));
  }
  m = block_reduce(m, true);
  if (threadIdx.x == 0) *out = m;
}

__global__ void k_ns_finish(int n, const double* __restrict__ g, const double* __restrict__ Z, double* __restrict__ X) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  X[(long)i * n + j] = Z[(long)i * n + j] / sqrt(g[1]);
}

// S^(-1/2) by the coupled Newton-Schulz iteration (Higham, "Functions of
// Matrices", 2008, eq. 6.35): Y0 = S/c, Z0 = I, M = 3I - Z Y,
// Y <- Y M / 2, Z <- M Z / 2; Z -> (S/c)^(-1/2).  c bounds the spectrum
// (Gershgorin), so S/c has eigenvalues in (0, 1].
gbhf_status inv_sqrt_dev(gbhf_ctx* c, int n, const double* d_S, double* d_X, int* iters) {
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, Y, 10, nn);
  GBHF_WS(c, Z, 11, nn);
  GBHF_WS(c, T, 12, nn);
  GBHF_WS(c, M, 23, nn);
  GBHF_CUDA(c, c->small.alloc(64));
  double* g = c->small.p + 32;
  double* e = c->small.p + 44;
  k_gershgorin<<<1, 1024, 0, c->stream>>>(n, d_S, g);
  k_ns_init<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, d_S, g, Y, Z);
  count_launch(c, 2);
  double err = 1;
  int it = 0;
  for (; it < 100; ++it) {
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, Z, n, Y, n, 0.0, T, n));
    if (it % 3 == 2) {
      k_ns_err<<<1, 1024, 0, c->stream>>>(n, T, e);
      count_launch(c);
      GBHF_CUDA(c, cudaMemcpyAsync(&err, e, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
      if (err < 1e-14) break;
    }
    k_three_minus<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, T, M);
    count_launch(c);
    GBHF_TRY(gemm(c, false, false, n, n, n, 0.5, Y, n, M, n, 0.0, T, n));
    std::swap(Y, T);
    GBHF_TRY(gemm(c, false, false, n, n, n, 0.5, M, n, Z, n, 0.0, T, n));
    std::swap(Z, T);
  }
  if (iters) *iters = it;
  if (!(err < 1e-10)) return fail(c, GBHF_ERR_NOT_CONVERGED, "Newton-Schulz S^-1/2 did not converge");
  k_ns_finish<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, g, Z, d_X);
  count_launch(c);
  return GBHF_OK;
}

// X = U s^-1/2 U^T (symmOrtho, HartreeFock/BasisOrthogonalization.hs:26-34)
__global__ void k_scale_cols(int n, const double* __restrict__ U, const double* __restrict__ s, double* __restrict__ out) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  out[(long)i * n + j] = U[(long)i * n + j] * (1.0 / sqrt(s[j]));
}

gbhf_status symm_ortho_dev(gbhf_ctx* c, int n, const double* d_S, double* d_X) {
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, U, 10, nn);
  GBHF_WS(c, s, 11, (size_t)n);
  GBHF_WS(c, T, 12, nn);
  GBHF_TRY(eigh(c, n, d_S, s, U, nullptr));
  k_scale_cols<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, U, s, T);
  count_launch(c);
  GBHF_TRY(gemm(c, false, true, n, n, n, 1.0, T, n, U, n, 0.0, d_X, n));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

// diagonalHF (HartreeFock/HartreeFock.hs:263-273) with square F in:
// F' = X^T F X, eigen-solve (warm-started from d_Cp when given; d_Cp receives
// the new C'), C = X C', D = 2 C_occ C_occ^T (calcDensity, :195-208).
gbhf_status diagonal_hf_dev(gbhf_ctx* c, int n, const double* d_Fsq, const double* d_X, int nocc, double* d_C,
                            double* d_Dsq, double* d_eps, double* d_Cp) {
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, T1, 10, nn);
  GBHF_WS(c, Fp, 11, nn);
  GBHF_WS(c, Cp, 12, nn);
  GBHF_TRY(gemm(c, true, false, n, n, n, 1.0, d_X, n, d_Fsq, n, 0.0, T1, n));
  GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, T1, n, d_X, n, 0.0, Fp, n, true));
  GBHF_TRY(eigh(c, n, Fp, d_eps, Cp, d_Cp));
  if (d_Cp) GBHF_CUDA(c, cudaMemcpyAsync(d_Cp, Cp, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, d_X, n, Cp, n, 0.0, d_C, n));
  if (nocc > 0) {
    GBHF_TRY(gemm(c, false, true, n, n, nocc, 2.0, d_C, n, d_C, n, 0.0, d_Dsq, n));
  } else {
    GBHF_CUDA(c, cudaMemsetAsync(d_Dsq, 0, nn * sizeof(double), c->stream));
  }
  return GBHF_OK;
}

// calcErrorMtx (HartreeFock/DIIS.hs:119-132): e = X^T (F D S - S D F) X, with
// S D F = (F D S)^T for symmetric F, D, S.
gbhf_status diis_error_dev(gbhf_ctx* c, int n, const double* d_F, const double* d_S, const double* d_D,
                           const double* d_X, double* d_e) {
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, T1, 13, nn);
  GBHF_WS(c, T2, 14, nn);
  GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, d_D, n, d_S, n, 0.0, T1, n));   // DS
  GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, d_F, n, T1, n, 0.0, T2, n));    // FDS
  k_antisym<<<dim3((n + 127) / 128, n), 128, 0, c->stream>>>(n, T2, T1);         // FDS - SDF
  count_launch(c);
  GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, T1, n, d_X, n, 0.0, T2, n));    // e X
  GBHF_TRY(gemm(c, true, false, n, n, n, 1.0, d_X, n, T2, n, 0.0, d_e, n));    // X^T e X
  return GBHF_OK;
}

}  // namespace gbhf
