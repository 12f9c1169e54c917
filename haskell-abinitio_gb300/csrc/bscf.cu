// Batched SCF: many molecules of uneven size advance together, each step one
// set of launches for all of them.
//
// The context's basis holds every molecule (atoms and functions contiguous
// per molecule); no shell pair or quartet spans two molecules.  Per-molecule
// square matrices are stacked: molecule m owns an n_m x n_m block at moff[m].
// A step of the batch is the step of scfDIIS (HartreeFock/HartreeFock.hs:
// 104-123) in the exact mode of scf.cu, for all molecules at once:
//   * the J/K build is the single-molecule build (the kernels take each
//     task's molecule from its bra pair), one launch per quartet class;
//   * the dense steps (DIIS error, orthogonalisation, trace-correcting purification,
//     Newton-Schulz S^-1/2) are grouped DMMA GEMMs whose CTAs each own one
//     16 x 16 tile of one molecule's block;
//   * per-molecule scalars (DIIS dot products, energies, convergence) come back
//     to the host in one read per step; the DIIS linear systems are solved on
//     the device, one thread per molecule.
// A molecule that has converged stops taking part: its quartets are dropped
// from the task lists and the dense kernels skip its block.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "dense.cuh"
#include "gbhf_internal.h"

namespace gbhf {

namespace {

constexpr int BMAX_DIIS = 8;   // DIIS vectors per molecule (current + stored)

struct BDesc {
  int M;
  const int* n;            // functions per molecule
  const long long* off;    // block offsets
  const int* tstart;       // first 16 x 16 tile of each molecule (M + 1)
  const int* active;       // per molecule 0/1
};

__device__ __forceinline__ int bd_mol(const int* tstart, int M, int x) {
  int lo = 0, hi = M - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tstart[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// 16 x 16 output tiles: with the batch's small blocks, 32 x 32 tiles carried 1.83x the
// symmetric product's flops in padding, 16 x 16 tiles 1.41x
constexpr int BT = 16, BKK = 16;
constexpr int WT = BT / 2, NI = WT / 8;   // per-warp tile (2 x 2 warps), 8 x 8 DMMA tiles per warp side

// C_m = alpha op(A_m) op(B_m) + beta C_m for every active molecule; one 32 x 32
// tile of one molecule's C per CTA (4 warps of 16 x 16, 2 x 2 DMMA tiles each).
// C must not alias A or B.  sym (C_m symmetric, beta = 0): tiles below the
// diagonal return at once and each tile above it is stored at its mirror too.
__global__ void __launch_bounds__(128) k_bgemm(BDesc d, int ta, int tb, int sym, double alpha,
                                               const double* __restrict__ A, const double* __restrict__ B,
                                               double beta, double* __restrict__ C) {
  const int m = bd_mol(d.tstart, d.M, blockIdx.x);
  if (!d.active[m]) return;
  const int n = d.n[m];
  const long long o = d.off[m];
  const int nt = (n + BT - 1) / BT, t = blockIdx.x - d.tstart[m];
  const int rt = t / nt, ct = t % nt;
  if (sym && rt > ct) return;
  const int row0 = rt * BT, col0 = ct * BT;
  const double* Am = A + o;
  const double* Bm = B + o;
  double* Cm = C + o;
  __shared__ double As[BT][BKK + 1];
  __shared__ double Bs[BKK][BT + 2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wr = (warp >> 1) * WT, wc = (warp & 1) * WT;
  double acc[NI][NI][2] = {};
  for (int kk = 0; kk < n; kk += BKK) {
    for (int idx = tid; idx < BT * BKK; idx += 128) {
      int r, cc;
      if (!ta) {
        r = idx / BKK;
        cc = idx % BKK;
      } else {
        cc = idx / BT;
        r = idx % BT;
      }
      const int gr = row0 + r, gk = kk + cc;
      double v = 0.0;
      if (gr < n && gk < n) v = ta ? Am[(long)gk * n + gr] : Am[(long)gr * n + gk];
      As[r][cc] = v;
    }
    for (int idx = tid; idx < BKK * BT; idx += 128) {
      int r, cc;
      if (!tb) {
        r = idx / BT;
        cc = idx % BT;
      } else {
        cc = idx / BKK;
        r = idx % BKK;
      }
      const int gk = kk + r, gc = col0 + cc;
      double v = 0.0;
      if (gk < n && gc < n) v = tb ? Bm[(long)gc * n + gk] : Bm[(long)gk * n + gc];
      Bs[r][cc] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k4 = 0; k4 < BKK; k4 += 4) {
      double af[NI], bf[NI];
#pragma unroll
      for (int i = 0; i < NI; ++i) af[i] = As[wr + i * 8 + (lane >> 2)][k4 + (lane & 3)];
#pragma unroll
      for (int j = 0; j < NI; ++j) bf[j] = Bs[k4 + (lane & 3)][wc + j * 8 + (lane >> 2)];
#pragma unroll
      for (int i = 0; i < NI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j) dmma(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < NI; ++i)
#pragma unroll
    for (int j = 0; j < NI; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = row0 + wr + i * 8 + (lane >> 2);
        const int cc = col0 + wc + j * 8 + 2 * (lane & 3) + h;
        if (r < n && cc < n) {
          double* p = Cm + (long)r * n + cc;
          *p = alpha * acc[i][j][h] + (beta == 0.0 ? 0.0 : beta * *p);
          if (sym && rt < ct) Cm[(long)cc * n + r] = alpha * acc[i][j][h];
        }
      }
}

// Elementwise kernels: grid (ceil(nmax^2 / 256), M), element (i, j) of molecule
// blockIdx.y.
#define BD_ELEMENT                                                  \
  const int m = blockIdx.y;                                         \
  if (!d.active[m]) return;                                         \
  const int n = d.n[m];                                             \
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;            \
  if (idx >= n * n) return;                                         \
  const int i = idx / n, j = idx - i * n;                           \
  const long long o = d.off[m];                                     \
  (void)i;                                                          \
  (void)j

// out = base + G + G^T (base may be nullptr or alias out)
__global__ void k_b_addsym(BDesc d, const double* base, const double* __restrict__ G, double* out) {
  BD_ELEMENT;
  const double v = G[o + (long)i * n + j] + G[o + (long)j * n + i];
  out[o + idx] = (base ? base[o + idx] : 0.0) + v;
}

// E = T - T^T
__global__ void k_b_antisym(BDesc d, const double* __restrict__ T, double* __restrict__ E) {
  BD_ELEMENT;
  E[o + idx] = T[o + (long)i * n + j] - T[o + (long)j * n + i];
}

// Newton-Schulz start: Y = S / c_m, Z = I (c_m = Gershgorin upper bound of S_m)
__global__ void k_b_ns_init(BDesc d, const double* __restrict__ S, const double* __restrict__ g, double* __restrict__ Y,
                            double* __restrict__ Z) {
  BD_ELEMENT;
  Y[o + idx] = S[o + idx] / g[4 * m + 1];
  Z[o + idx] = i == j ? 1.0 : 0.0;
}

__global__ void k_b_three_minus(BDesc d, const double* __restrict__ T, double* __restrict__ Mo) {
  BD_ELEMENT;
  Mo[o + idx] = (i == j ? 3.0 : 0.0) - T[o + idx];
}

__global__ void k_b_ns_finish(BDesc d, const double* __restrict__ g, const double* __restrict__ Z,
                              double* __restrict__ X) {
  BD_ELEMENT;
  X[o + idx] = Z[o + idx] / sqrt(g[4 * m + 1]);
}

// Canonical purification start (Palser & Manolopoulos 1998):
// P = lambda/n (mu I - F) + ne/n I, mu = tr F / n.
__global__ void k_b_purify_init(BDesc d, const int* __restrict__ ne, const double* __restrict__ F,
                                const double* __restrict__ g, double* __restrict__ P) {
  BD_ELEMENT;
  const double lo = g[4 * m], hi = g[4 * m + 1], mu = g[4 * m + 2] / n;
  const int e = ne[m];
  double lam = 1e300;
  if (hi - mu > 0) lam = fmin(lam, e / (hi - mu));
  if (mu - lo > 0) lam = fmin(lam, (n - e) / (mu - lo));
  if (!(lam < 1e300)) lam = 0;
  P[o + idx] = (lam / n) * ((i == j ? mu : 0.0) - F[o + idx]) + (i == j ? (double)e / n : 0.0);
}

__global__ void k_b_purify_update(BDesc d, const double* __restrict__ coef, double* __restrict__ P,
                                  const double* __restrict__ P2, const double* __restrict__ P3) {
  BD_ELEMENT;
  const double* c = coef + 4 * m;
  P[o + idx] = c[0] * P[o + idx] + c[1] * P2[o + idx] + c[2] * P3[o + idx];
}

// Per-molecule reductions: one block per molecule.
// Gershgorin bounds and trace of A_m: g[4m] = lo, g[4m+1] = hi, g[4m+2] = trace.
__global__ void k_b_gershgorin(BDesc d, const double* __restrict__ A, double* __restrict__ g) {
  const int m = blockIdx.x;
  if (!d.active[m]) return;
  const int n = d.n[m];
  const double* Am = A + d.off[m];
  double lo = 1e300, hi = -1e300, tr = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double r = 0;
    for (int j = 0; j < n; ++j)
      if (j != i) r += fabs(Am[(long)i * n + j]);
    lo = fmin(lo, Am[(long)i * n + i] - r);
    hi = fmax(hi, Am[(long)i * n + i] + r);
    tr += Am[(long)i * n + i];
  }
  // min / max / sum over the block (identities +-1e300, 0)
  __shared__ double s_lo[32], s_hi[32], s_tr[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    tr += __shfl_xor_sync(0xffffffffu, tr, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
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
    g[4 * m] = lo;
    g[4 * m + 1] = hi;
    g[4 * m + 2] = tr;
  }
}

// max |T - I| per molecule
__global__ void k_b_maxdev_identity(BDesc d, const double* __restrict__ T, double* __restrict__ out) {
  const int m = blockIdx.x;
  if (!d.active[m]) return;
  const int n = d.n[m];
  const double* Tm = T + d.off[m];
  double v = 0;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - i * n;
    v = fmax(v, fabs(Tm[idx] - (i == j ? 1.0 : 0.0)));
  }
  v = block_reduce(v, true);
  if (threadIdx.x == 0) out[m] = v;
}

// traces of P, P^2, P^3 -> next purification polynomial, coef[4m] = (a, b, c, tr(P - P^2));
// a molecule whose idempotency error is below tol * nocc leaves the purification
// (its flag in d.active, a copy of the batch's flags, is cleared)
__global__ void k_b_purify_coef(BDesc d, const double* __restrict__ P, const double* __restrict__ P2,
                                const double* __restrict__ P3, double* __restrict__ coef,
                                const int* __restrict__ nocc, double tol, int* __restrict__ pact) {
  const int m = blockIdx.x;
  if (!d.active[m]) return;
  const int n = d.n[m];
  const long long o = d.off[m];
  double t1 = 0, t2 = 0, t3 = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    t1 += P[o + (long)i * n + i];
    t2 += P2[o + (long)i * n + i];
    t3 += P3[o + (long)i * n + i];
  }
  t1 = block_reduce(t1, false);
  __syncthreads();
  t2 = block_reduce(t2, false);
  __syncthreads();
  t3 = block_reduce(t3, false);
  if (threadIdx.x == 0) {
    const double den = t1 - t2, num = t2 - t3;
    double a = 1, b = 0, c = 0;
    if (fabs(den) > 1e-300) {
      const double cc = num / den;
      if (cc >= 0.5) {
        a = 0;
        b = (1 + cc) / cc;
        c = -1 / cc;
      } else {
        a = (1 - 2 * cc) / (1 - cc);
        b = (1 + cc) / (1 - cc);
        c = -1 / (1 - cc);
      }
    }
    coef[4 * m] = a;
    coef[4 * m + 1] = b;
    coef[4 * m + 2] = c;
    coef[4 * m + 3] = den;
    if (fabs(den) < tol * (double)max(1, nocc[m])) pact[m] = 0;   // P meets the tolerance: no further update
  }
}

// TC2 purification (one GEMM per step): start P = (hi I - F) / (hi - lo), then
// P <- P^2 or 2P - P^2, whichever moves tr P toward nocc.
__global__ void k_b_tc2_init(BDesc d, const double* __restrict__ F, const double* __restrict__ g,
                             double* __restrict__ P) {
  BD_ELEMENT;
  const double lo = g[4 * m], hi = g[4 * m + 1];
  const double sc = hi > lo ? 1.0 / (hi - lo) : 0.0;
  P[o + idx] = sc * ((i == j ? hi : 0.0) - F[o + idx]);
}

// traces of P and P^2 -> coef[4m] = (a, b, 0, tr(P - P^2)) of P' = a P + b P^2;
// converged molecules leave as in k_b_purify_coef
__global__ void k_b_tc2_coef(BDesc d, const double* __restrict__ P, const double* __restrict__ P2,
                             double* __restrict__ coef, const int* __restrict__ nocc, double tol,
                             int* __restrict__ pact) {
  const int m = blockIdx.x;
  if (!d.active[m]) return;
  const int n = d.n[m];
  const long long o = d.off[m];
  double t1 = 0, t2 = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    t1 += P[o + (long)i * n + i];
    t2 += P2[o + (long)i * n + i];
  }
  t1 = block_reduce(t1, false);
  __syncthreads();
  t2 = block_reduce(t2, false);
  if (threadIdx.x == 0) {
    const double den = t1 - t2, ne = (double)nocc[m];
    const bool sq = fabs(t2 - ne) < fabs(2 * t1 - t2 - ne);
    coef[4 * m] = sq ? 0.0 : 2.0;
    coef[4 * m + 1] = sq ? 1.0 : -1.0;
    coef[4 * m + 2] = 0.0;
    coef[4 * m + 3] = den;
    if (fabs(den) < tol * (double)max(1, nocc[m])) pact[m] = 0;
  }
}

struct HistPtrs {
  double* p[BMAX_DIIS];
};

// DIIS dot products: out[BMAX_DIIS*m + j] = <E_m, hist[slot(m, j)]_m> for the
// molecule's stored slots (newest first), out[BMAX_DIIS*m + k] = <E_m, E_m>,
// and emax[m] = max |E_m|.
__global__ void k_b_dots(BDesc d, const double* __restrict__ E, HistPtrs hist, const int* __restrict__ slots,
                         const int* __restrict__ nstored, double* __restrict__ out, double* __restrict__ emax) {
  const int m = blockIdx.x;
  if (!d.active[m]) return;
  const int n = d.n[m];
  const long long o = d.off[m];
  const int k = nstored[m];
  for (int j = 0; j <= k; ++j) {
    const double* H = j < k ? hist.p[slots[BMAX_DIIS * m + j]] + o : E + o;
    double s = 0;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) s += E[o + idx] * H[idx];
    s = block_reduce(s, false);
    if (threadIdx.x == 0) out[BMAX_DIIS * m + j] = s;
    __syncthreads();
  }
  double mx = 0;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) mx = fmax(mx, fabs(E[o + idx]));
  mx = block_reduce(mx, true);
  if (threadIdx.x == 0) emax[m] = mx;
}

// gaussElem for every molecule with a system (size > 0): thread per molecule.
__global__ void k_b_gauss(int M, const int* __restrict__ size, const double* __restrict__ a_in,
                          const double* __restrict__ b_in, double* __restrict__ x, int* __restrict__ ok) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const int s = size[m];
  if (s <= 0) return;
  double a[(BMAX_DIIS + 1) * (BMAX_DIIS + 1)], b[BMAX_DIIS + 1];
  for (int i = 0; i < s * s; ++i) a[i] = a_in[(BMAX_DIIS + 1) * (BMAX_DIIS + 1) * m + i];
  for (int i = 0; i < s; ++i) b[i] = b_in[(BMAX_DIIS + 1) * m + i];
  ok[m] = gauss_elem_dev(s, a, b, x + (BMAX_DIIS + 1) * m) ? 1 : 0;
}

// Fd_m = c_0 F_m + sum_j c_(j+1) hist[slot(m, j)]_m
__global__ void k_b_lincomb(BDesc d, const double* __restrict__ F, HistPtrs hist, const int* __restrict__ slots,
                            const int* __restrict__ nterm, const double* __restrict__ coef, double* __restrict__ out) {
  BD_ELEMENT;
  const int k = nterm[m];
  const double* c = coef + BMAX_DIIS * m;
  double s = c[0] * F[o + idx];
  for (int j = 1; j < k; ++j) s += c[j] * hist.p[slots[BMAX_DIIS * m + j - 1]][o + idx];
  out[o + idx] = s;
}

// copy E_m, F_m into history slot slot[m] (molecules with slot >= 0)
__global__ void k_b_store(BDesc d, const double* __restrict__ E, const double* __restrict__ F, HistPtrs he,
                          HistPtrs hf, const int* __restrict__ slot) {
  BD_ELEMENT;
  const int s = slot[m];
  if (s < 0) return;
  he.p[s][o + idx] = E[o + idx];
  hf.p[s][o + idx] = F[o + idx];
}

// E[D] = 1/2 sum D (H + F) and sum (Dn - D)^2 per molecule
__global__ void k_b_stats(BDesc d, const double* __restrict__ H, const double* __restrict__ F,
                          const double* __restrict__ D, const double* __restrict__ Dn, double* __restrict__ out) {
  const int m = blockIdx.x;
  if (!d.active[m]) return;
  const int n = d.n[m];
  const long long o = d.off[m];
  double en = 0, dd = 0;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    en += D[o + idx] * (H[o + idx] + F[o + idx]);
    const double x = Dn[o + idx] - D[o + idx];
    dd += x * x;
  }
  en = block_reduce(en, false);
  __syncthreads();
  dd = block_reduce(dd, false);
  if (threadIdx.x == 0) {
    out[2 * m] = 0.5 * en;
    out[2 * m + 1] = dd;
  }
}

#undef BD_ELEMENT

}  // namespace

// Host side of the batch: layout, work matrices, per-molecule DIIS state.
struct BatchRun {
  gbhf_ctx* c;
  int M = 0, nmax = 0, ntiles = 0;
  size_t nst = 0;
  std::vector<int> n, tstart, nocc, active;
  std::vector<long long> off;
  DBuf<int> d_n, d_tstart, d_active, d_nocc, d_pact;
  DBuf<long long> d_off;
  BDesc desc{};

  gbhf_status init(gbhf_ctx* cc, const std::vector<int>& occ) {
    c = cc;
    const Basis& b = c->basis;
    M = b.nmol;
    n.resize(M);
    off.assign(b.mol_moff.begin(), b.mol_moff.begin() + M);
    tstart.resize(M + 1);
    tstart[0] = 0;
    for (int m = 0; m < M; ++m) {
      n[m] = b.mol_fn_off[m + 1] - b.mol_fn_off[m];
      nmax = std::max(nmax, n[m]);
      const int nt = (n[m] + BT - 1) / BT;
      tstart[m + 1] = tstart[m] + nt * nt;
    }
    ntiles = tstart[M];
    nst = (size_t)b.stacked;
    nocc = occ;
    active.assign(M, 1);
    GBHF_CUDA(c, d_n.alloc(M));
    GBHF_CUDA(c, d_off.alloc(M));
    GBHF_CUDA(c, d_tstart.alloc(M + 1));
    GBHF_CUDA(c, d_active.alloc(M));
    GBHF_CUDA(c, d_nocc.alloc(M));
    GBHF_CUDA(c, cudaMemcpyAsync(d_n.p, n.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(d_off.p, off.data(), M * sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(d_tstart.p, tstart.data(), (M + 1) * sizeof(int), cudaMemcpyHostToDevice,
                                 c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(d_nocc.p, nocc.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GBHF_TRY(set_active(active));
    desc.M = M;
    desc.n = d_n.p;
    desc.off = d_off.p;
    desc.tstart = d_tstart.p;
    desc.active = d_active.p;
    return GBHF_OK;
  }
  gbhf_status set_active(const std::vector<int>& a) {
    active = a;
    GBHF_CUDA(c, cudaMemcpyAsync(d_active.p, active.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    return GBHF_OK;
  }
  dim3 egrid() const { return dim3((unsigned)((nmax * nmax + 255) / 256), (unsigned)M); }
  // sym: every C_m is symmetric (beta must be 0); dsc: other per-molecule active flags
  gbhf_status gemm(bool ta, bool tb, double alpha, const double* A, const double* B, double beta, double* C,
                   bool sym = false, const BDesc* dsc = nullptr) {
    k_bgemm<<<ntiles, 128, 0, c->stream>>>(dsc ? *dsc : desc, ta, tb, sym && beta == 0.0 ? 1 : 0, alpha, A, B, beta,
                                           C);
    count_launch(c);
    GBHF_CUDA(c, cudaGetLastError());
    return GBHF_OK;
  }
};

namespace {

// S^(-1/2) of every molecule by the coupled Newton-Schulz iteration (as inv_sqrt_dev).
gbhf_status b_inv_sqrt(BatchRun& br, const double* S, double* X, double* Y, double* Z, double* T, double* Mw,
                       double* g, double* e) {
  gbhf_ctx* c = br.c;
  k_b_gershgorin<<<br.M, 256, 0, c->stream>>>(br.desc, S, g);
  k_b_ns_init<<<br.egrid(), 256, 0, c->stream>>>(br.desc, S, g, Y, Z);
  count_launch(c, 2);
  std::vector<double> err(br.M);
  bool done = false;
  for (int it = 0; it < 100 && !done; ++it) {
    GBHF_TRY(br.gemm(false, false, 1.0, Z, Y, 0.0, T));
    if (it % 3 == 2) {
      k_b_maxdev_identity<<<br.M, 256, 0, c->stream>>>(br.desc, T, e);
      count_launch(c);
      GBHF_CUDA(c, cudaMemcpyAsync(err.data(), e, br.M * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
      done = true;
      for (int m = 0; m < br.M; ++m)
        if (br.active[m] && !(err[m] < 1e-14)) done = false;
      if (done) break;
    }
    k_b_three_minus<<<br.egrid(), 256, 0, c->stream>>>(br.desc, T, Mw);
    count_launch(c);
    GBHF_TRY(br.gemm(false, false, 0.5, Y, Mw, 0.0, T));
    std::swap(Y, T);
    GBHF_TRY(br.gemm(false, false, 0.5, Mw, Z, 0.0, T));
    std::swap(Z, T);
  }
  for (int m = 0; m < br.M; ++m)
    if (br.active[m] && !(err[m] < 1e-10))
      return fail(c, GBHF_ERR_NOT_CONVERGED, "Newton-Schulz S^-1/2 did not converge for molecule " + std::to_string(m));
  k_b_ns_finish<<<br.egrid(), 256, 0, c->stream>>>(br.desc, g, Z, X);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// D_m = X_m (2 P_m) X_m^T with P_m the projector onto the nocc_m lowest
// eigenvectors of X_m^T F_m X_m (trace-correcting purification, as density_purified_dev).
gbhf_status b_density(BatchRun& br, const double* F, const double* X, double* D, double* T1, double* Fp, double* P,
                      double* P2, double* P3, double* g, double* coef) {
  gbhf_ctx* c = br.c;
  GBHF_TRY(br.gemm(true, false, 1.0, X, F, 0.0, T1));
  GBHF_TRY(br.gemm(false, false, 1.0, T1, X, 0.0, Fp, true));
  // trace-correcting purification: a third fewer GEMMs than the canonical one
  // on water clusters (see purify in linalg.cu)
  constexpr bool tc2 = true;
  k_b_gershgorin<<<br.M, 256, 0, c->stream>>>(br.desc, Fp, g);
  if (tc2) k_b_tc2_init<<<br.egrid(), 256, 0, c->stream>>>(br.desc, Fp, g, P);
  else k_b_purify_init<<<br.egrid(), 256, 0, c->stream>>>(br.desc, br.d_nocc.p, Fp, g, P);
  count_launch(c, 2);
  std::vector<double> hc(4 * (size_t)br.M);
  // molecules still purifying: a copy of the active flags that k_b_purify_coef clears
  GBHF_CUDA(c, br.d_pact.alloc(br.M));
  GBHF_CUDA(c, cudaMemcpyAsync(br.d_pact.p, br.d_active.p, br.M * sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
  BDesc pd = br.desc;
  pd.active = br.d_pact.p;
  const double tol = 1e-13;
  // four purification steps per CUDA-graph replay, convergence read between replays
  auto four_steps = [&]() -> gbhf_status {
    for (int k = 0; k < 4; ++k) {
      GBHF_TRY(br.gemm(false, false, 1.0, P, P, 0.0, P2, true, &pd));
      if (tc2) {
        k_b_tc2_coef<<<br.M, 256, 0, c->stream>>>(pd, P, P2, coef, br.d_nocc.p, tol, br.d_pact.p);
        k_b_purify_update<<<br.egrid(), 256, 0, c->stream>>>(pd, coef, P, P2, P2);   // third coefficient 0
        count_launch(c, 2);
        continue;
      }
      GBHF_TRY(br.gemm(false, false, 1.0, P, P2, 0.0, P3, true, &pd));
      k_b_purify_coef<<<br.M, 256, 0, c->stream>>>(pd, P, P2, P3, coef, br.d_nocc.p, tol, br.d_pact.p);
      k_b_purify_update<<<br.egrid(), 256, 0, c->stream>>>(pd, coef, P, P2, P3);
      count_launch(c, 2);
    }
    return GBHF_OK;
  };
  const std::vector<const void*> key = {(const void*)(size_t)br.M, (const void*)(size_t)br.ntiles,
                                        (const void*)(size_t)br.nmax, br.desc.n, br.desc.off, br.desc.tstart,
                                        br.d_pact.p, br.d_nocc.p, P, P2, P3, coef};
  bool done = false;
  for (int rep = 0; rep < 50 && !done; ++rep) {
    GBHF_TRY(graph_run(c, c->g_bpurify, key, four_steps));
    GBHF_CUDA(c, cudaMemcpyAsync(hc.data(), coef, hc.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    done = true;
    for (int m = 0; m < br.M; ++m)
      if (br.active[m] && !(std::fabs(hc[4 * m + 3]) < tol * std::max(1, br.nocc[m]))) done = false;
  }
  for (int m = 0; m < br.M; ++m)
    if (br.active[m] && !(std::fabs(hc[4 * m + 3]) < 1e-6 * std::max(1, br.nocc[m])))
      return fail(c, GBHF_ERR_NOT_CONVERGED, "density purification did not converge for molecule " + std::to_string(m));
  GBHF_TRY(br.gemm(false, false, 2.0, X, P, 0.0, T1));
  GBHF_TRY(br.gemm(false, true, 1.0, T1, X, 0.0, D, true));
  return GBHF_OK;
}

// Per-molecule DIIS history (DIIS.hs:55-114), as the single-molecule driver.
struct MolDiis {
  std::vector<int> stored;                    // slots, newest first
  std::vector<int> free_slots;
  std::vector<std::vector<double>> Bst;       // dots among stored (newest first)
  bool on = false;
};

}  // namespace

gbhf_status bscf_run(gbhf_ctx* c, const gbhf_scf_opts* o, double* energies, int* iterations, int* converged_out,
                     double* grads) {
  const Basis& b = c->basis;
  const int M = b.nmol;
  if (o->mode != GBHF_MODE_EXACT) return fail(c, GBHF_ERR_UNSUPPORTED, "batched SCF runs the exact mode");
  if (o->diis_size < 1 || o->diis_size > BMAX_DIIS - 1)
    return fail(c, GBHF_ERR_BAD_INPUT, "batched SCF: diis_size must be 1..7");
  if (o->max_iter < 1) return fail(c, GBHF_ERR_BAD_INPUT, "max_iter must be >= 1");
  GBHF_TRY(ensure_boys_tables(c));
  GBHF_TRY(ensure_pairs(c));
  GBHF_TRY(ensure_shell_arrays(c));
  std::vector<int> nocc(M);
  std::vector<double> enuc(M, 0.0);
  for (int m = 0; m < M; ++m) {
    double zsum = 0;
    const int a0 = b.mol_atom_off[m], a1 = b.mol_atom_off[m + 1];
    for (int a = a0; a < a1; ++a) zsum += b.Z[a];
    nocc[m] = (int)std::floor((zsum - o->charge) / 2.0);
    const int nm = b.mol_fn_off[m + 1] - b.mol_fn_off[m];
    if (nocc[m] < 0 || nocc[m] > nm)
      return fail(c, GBHF_ERR_BAD_INPUT, "molecule " + std::to_string(m) + ": occupied orbitals out of range");
    for (int a = a0; a < a1; ++a)
      for (int a2 = a + 1; a2 < a1; ++a2) {
        double r2 = 0;
        for (int x = 0; x < 3; ++x) r2 += (b.xyz[3 * a + x] - b.xyz[3 * a2 + x]) * (b.xyz[3 * a + x] - b.xyz[3 * a2 + x]);
        enuc[m] += b.Z[a] * b.Z[a2] / std::sqrt(r2);
      }
  }
  using clk = std::chrono::steady_clock;
  auto ms_since = [](clk::time_point t0) {
    return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
  };
  auto t_phase = clk::now();
  BatchRun br;
  GBHF_TRY(br.init(c, nocc));
  const size_t nst = br.nst;
  // stacked work matrices
  const int maxstore = o->diis_size - 1;
  const int NW = 20;
  std::vector<DBuf<double>> wb(NW + 2 * (maxstore + 1));
  for (auto& w : wb) GBHF_CUDA(c, w.alloc(std::max<size_t>(nst, 1)));
  double *S = wb[0].p, *H = wb[1].p, *X = wb[2].p, *D = wb[3].p, *Dn = wb[4].p, *F = wb[5].p, *Fd = wb[6].p,
         *Gacc = wb[7].p, *Gpp = wb[8].p, *E = wb[9].p, *Dref = wb[10].p, *T1 = wb[11].p, *T2 = wb[12].p,
         *P = wb[13].p, *P2 = wb[14].p, *P3 = wb[15].p, *Fp = wb[16].p, *Ffin = wb[17].p, *Wm = wb[18].p,
         *Dg = wb[19].p;
  HistPtrs he{}, hf{};
  for (int s = 0; s <= maxstore; ++s) {
    he.p[s] = wb[NW + 2 * s].p;
    hf.p[s] = wb[NW + 2 * s + 1].p;
  }
  DBuf<double> small;
  GBHF_CUDA(c, small.alloc(32 * (size_t)M + 64));
  double* d_g = small.p;                  // 4 per molecule
  double* d_coef = small.p + 4 * M;       // 4 per molecule
  double* d_err = small.p + 8 * M;        // 1 per molecule
  double* d_emax = small.p + 9 * M;       // 1 per molecule
  double* d_stats = small.p + 10 * M;     // 2 per molecule
  DBuf<double> d_dots, d_sys, d_rhs, d_x, d_lc;
  DBuf<int> d_slots, d_nst, d_size, d_ok, d_nterm, d_store;
  GBHF_CUDA(c, d_dots.alloc(BMAX_DIIS * (size_t)M));
  GBHF_CUDA(c, d_sys.alloc((BMAX_DIIS + 1) * (BMAX_DIIS + 1) * (size_t)M));
  GBHF_CUDA(c, d_rhs.alloc((BMAX_DIIS + 1) * (size_t)M));
  GBHF_CUDA(c, d_x.alloc((BMAX_DIIS + 1) * (size_t)M));
  GBHF_CUDA(c, d_lc.alloc(BMAX_DIIS * (size_t)M));
  GBHF_CUDA(c, d_slots.alloc(BMAX_DIIS * (size_t)M));
  GBHF_CUDA(c, d_nst.alloc(M));
  GBHF_CUDA(c, d_size.alloc(M));
  GBHF_CUDA(c, d_ok.alloc(M));
  GBHF_CUDA(c, d_nterm.alloc(M));
  GBHF_CUDA(c, d_store.alloc(M));

  // one-electron matrices, orthogonaliser, SAD start
  GBHF_TRY(onee_stacked(c, S, H));
  GBHF_TRY(b_inv_sqrt(br, S, X, T1, T2, P, P2, d_g, d_err));
  if (o->guess == GBHF_GUESS_SAD) {
    GBHF_TRY(sad_density(c, D));
  } else if (o->guess == GBHF_GUESS_CORE) {
    GBHF_TRY(b_density(br, H, X, D, T1, Fp, P, P2, P3, d_g, d_coef));
  } else {
    return fail(c, GBHF_ERR_UNSUPPORTED, "batched SCF starts from the SAD or core guess");
  }
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->prof.ph_setup += ms_since(t_phase);
  if (o->autotune && !c->tuned[0]) {   // J/K budgets on this basis and starting density
    GBHF_TRY(autotune_dev(c, 0, D, o->precision, o->schwarz_cutoff,
                          o->precision == GBHF_PREC_FP64 ? 0.0 : o->mixed_cutoff, 2, nullptr));
  }
  std::vector<MolDiis> diis(M);
  for (auto& md : diis)
    for (int s = 0; s <= maxstore; ++s) md.free_slots.push_back(s);
  std::vector<double> e_prev(M, 0.0), energy(M, 0.0);
  std::vector<int> have_prev(M, 0), conv(M, 0), iters(M, 0);
  std::vector<double> hdots(BMAX_DIIS * (size_t)M), hemax(M), hstats(2 * (size_t)M);
  std::vector<int> hslots(BMAX_DIIS * (size_t)M), hnst(M), hsize(M), hok(M), hnterm(M), hstore(M);
  std::vector<double> hsys((BMAX_DIIS + 1) * (BMAX_DIIS + 1) * (size_t)M), hrhs((BMAX_DIIS + 1) * (size_t)M),
      hx((BMAX_DIIS + 1) * (size_t)M), hlc(BMAX_DIIS * (size_t)M);
  int precision = o->precision;
  bool fp64_final_phase = false;
  int since_full = 1 << 30;
  struct ActiveGuard {   // the J/K lists follow the active set only inside this call
    gbhf_ctx* c;
    ~ActiveGuard() {
      c->mol_active = nullptr;
      c->tasks.thr_all = -1;
    }
  } guard{c};
  c->mol_active = br.d_active.p;
  c->tasks.thr_all = -1;
  gbhf_status status = GBHF_OK;
  int step = 0;
  for (step = 0; step < o->max_iter; ++step) {
    // ---- Fock matrices of the current densities
    t_phase = clk::now();
    const bool full = !o->incremental ||
                      since_full >= (o->full_rebuild_every > 0 ? o->full_rebuild_every : (1 << 30)) || step == 0 ||
                      fp64_final_phase;
    GBHF_CUDA(c, cudaMemsetAsync(Gpp, 0, nst * sizeof(double), c->stream));
    if (full) {
      c->tasks.thr_all = -1;   // the active set may have changed since the cached lists
      status = jk_build(c, D, Gpp, precision, o->schwarz_cutoff, o->mixed_cutoff, 1.0);
      if (status != GBHF_OK) break;
      k_b_addsym<<<br.egrid(), 256, 0, c->stream>>>(br.desc, nullptr, Gpp, Gacc);
      since_full = 1;
    } else {
      GBHF_TRY(axpby(c, nst, 1.0, D, -1.0, Dref, Dn));   // dD (Dn as scratch)
      status = jk_build(c, Dn, Gpp, precision, o->schwarz_cutoff, o->mixed_cutoff, 1.0, true);
      if (status != GBHF_OK) break;
      k_b_addsym<<<br.egrid(), 256, 0, c->stream>>>(br.desc, Gacc, Gpp, Gacc);
      ++since_full;
    }
    count_launch(c);
    GBHF_CUDA(c, cudaMemcpyAsync(Dref, D, nst * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    GBHF_TRY(axpby(c, nst, 1.0, H, 1.0, Gacc, F));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->prof.ph_fock += ms_since(t_phase);
    t_phase = clk::now();
    // ---- DIIS error e = X^T (F D S - S D F) X and dot products
    GBHF_TRY(br.gemm(false, false, 1.0, F, D, 0.0, T1));
    GBHF_TRY(br.gemm(false, false, 1.0, T1, S, 0.0, T2));
    k_b_antisym<<<br.egrid(), 256, 0, c->stream>>>(br.desc, T2, T1);
    count_launch(c);
    GBHF_TRY(br.gemm(true, false, 1.0, X, T1, 0.0, T2));
    GBHF_TRY(br.gemm(false, false, 1.0, T2, X, 0.0, E));
    for (int m = 0; m < M; ++m) {
      hnst[m] = br.active[m] ? (int)diis[m].stored.size() : 0;
      for (int j = 0; j < hnst[m]; ++j) hslots[BMAX_DIIS * m + j] = diis[m].stored[j];
    }
    GBHF_CUDA(c, cudaMemcpyAsync(d_slots.p, hslots.data(), hslots.size() * sizeof(int), cudaMemcpyHostToDevice,
                                 c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(d_nst.p, hnst.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    k_b_dots<<<M, 256, 0, c->stream>>>(br.desc, E, he, d_slots.p, d_nst.p, d_dots.p, d_emax);
    count_launch(c);
    GBHF_CUDA(c, cudaMemcpyAsync(hdots.data(), d_dots.p, hdots.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                 c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(hemax.data(), d_emax, M * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    // ---- DIIS per molecule (diisDriver / diis / updateDIIS)
    std::vector<std::vector<double>> newdots(M);
    for (int m = 0; m < M; ++m) {
      if (!br.active[m]) continue;
      newdots[m].assign(hdots.begin() + BMAX_DIIS * m, hdots.begin() + BMAX_DIIS * m + hnst[m] + 1);
    }
    auto drop_oldest = [&](int m) {
      MolDiis& md = diis[m];
      md.free_slots.push_back(md.stored.back());
      md.stored.pop_back();
      md.Bst.pop_back();
      for (auto& row : md.Bst) row.pop_back();
      newdots[m].erase(newdots[m].end() - 2);
    };
    std::vector<int> extrap(M, 0);   // 1: extrapolate this step
    for (int m = 0; m < M; ++m) {
      hnterm[m] = 1;
      hlc[BMAX_DIIS * m] = 1.0;
      if (!br.active[m]) continue;
      if (diis[m].on) extrap[m] = 1;
    }
    // solve the systems; molecules whose system fails drop their oldest pair and retry
    while (true) {
      bool any = false;
      for (int m = 0; m < M; ++m) {
        hsize[m] = 0;
        if (!extrap[m] || extrap[m] == 2) continue;
        const MolDiis& md = diis[m];
        const int k = 1 + (int)md.stored.size();
        const int s = k + 1;
        double* A = hsys.data() + (BMAX_DIIS + 1) * (BMAX_DIIS + 1) * (size_t)m;
        double* r = hrhs.data() + (BMAX_DIIS + 1) * (size_t)m;
        const std::vector<double>& nd = newdots[m];
        for (int i = 0; i < s * s; ++i) A[i] = 0.0;
        for (int i = 0; i < k; ++i)
          for (int j = 0; j < k; ++j) {
            double v;
            if (i == 0 && j == 0) v = nd.back();
            else if (i == 0) v = nd[j - 1];
            else if (j == 0) v = nd[i - 1];
            else v = md.Bst[i - 1][j - 1];
            A[i * s + j] = v;
          }
        for (int i = 0; i < k; ++i) {
          A[i * s + k] = -1.0;
          A[k * s + i] = -1.0;
        }
        for (int i = 0; i < s; ++i) r[i] = 0.0;
        r[k] = -1.0;
        hsize[m] = s;
        any = true;
      }
      if (!any) break;
      GBHF_CUDA(c, cudaMemcpyAsync(d_sys.p, hsys.data(), hsys.size() * sizeof(double), cudaMemcpyHostToDevice,
                                   c->stream));
      GBHF_CUDA(c, cudaMemcpyAsync(d_rhs.p, hrhs.data(), hrhs.size() * sizeof(double), cudaMemcpyHostToDevice,
                                   c->stream));
      GBHF_CUDA(c, cudaMemcpyAsync(d_size.p, hsize.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
      k_b_gauss<<<(M + 127) / 128, 128, 0, c->stream>>>(M, d_size.p, d_sys.p, d_rhs.p, d_x.p, d_ok.p);
      count_launch(c);
      GBHF_CUDA(c, cudaMemcpyAsync(hx.data(), d_x.p, hx.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      GBHF_CUDA(c, cudaMemcpyAsync(hok.data(), d_ok.p, M * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
      for (int m = 0; m < M; ++m) {
        if (hsize[m] == 0) continue;
        const int k = hsize[m] - 1;
        if (hok[m]) {
          extrap[m] = 2;   // solved
          hnterm[m] = k;
          for (int j = 0; j < k; ++j) hlc[BMAX_DIIS * m + j] = hx[(BMAX_DIIS + 1) * (size_t)m + j];
          for (int j = 0; j + 1 < k; ++j) hslots[BMAX_DIIS * m + j] = diis[m].stored[j];
        } else {
          if (diis[m].stored.empty())
            return fail(c, GBHF_ERR_SINGULAR, "molecule " + std::to_string(m) + ": DIIS system singular");
          drop_oldest(m);
        }
      }
    }
    // new (e, F) pairs into the history: the ON branch always, the OFF branch
    // once max|e| drops below diis_start after the first step
    for (int m = 0; m < M; ++m) {
      hstore[m] = -1;
      if (!br.active[m] || maxstore == 0) continue;
      MolDiis& md = diis[m];
      const bool add = md.on || (step > 0 && hemax[m] < o->diis_start);
      if (!add) continue;
      if (!md.on) md.on = true;
      if ((int)md.stored.size() >= maxstore) drop_oldest(m);
      const int slot = md.free_slots.back();
      md.free_slots.pop_back();
      const std::vector<double>& nd = newdots[m];
      std::vector<double> row;
      row.push_back(nd.back());
      for (size_t j = 0; j < md.stored.size(); ++j) row.push_back(nd[j]);
      for (size_t i = 0; i < md.Bst.size(); ++i) md.Bst[i].insert(md.Bst[i].begin(), nd[i]);
      md.Bst.insert(md.Bst.begin(), row);
      md.stored.insert(md.stored.begin(), slot);
      hstore[m] = slot;
    }
    // extrapolated Fock (before the store overwrites a slot of the combination)
    GBHF_CUDA(c, cudaMemcpyAsync(d_slots.p, hslots.data(), hslots.size() * sizeof(int), cudaMemcpyHostToDevice,
                                 c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(d_nterm.p, hnterm.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(d_lc.p, hlc.data(), hlc.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    k_b_lincomb<<<br.egrid(), 256, 0, c->stream>>>(br.desc, F, hf, d_slots.p, d_nterm.p, d_lc.p, Fd);
    GBHF_CUDA(c, cudaMemcpyAsync(d_store.p, hstore.data(), M * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    k_b_store<<<br.egrid(), 256, 0, c->stream>>>(br.desc, E, F, he, hf, d_store.p);
    count_launch(c, 2);
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->prof.ph_diis += ms_since(t_phase);
    t_phase = clk::now();
    // ---- new densities
    status = b_density(br, Fd, X, Dn, T1, Fp, P, P2, P3, d_g, d_coef);
    if (status != GBHF_OK) break;
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->prof.ph_diag += ms_since(t_phase);
    t_phase = clk::now();
    // ---- energies and convergence
    k_b_stats<<<M, 256, 0, c->stream>>>(br.desc, H, F, D, Dn, d_stats);
    count_launch(c);
    GBHF_CUDA(c, cudaMemcpyAsync(hstats.data(), d_stats, hstats.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                 c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<int> act = br.active;
    bool any_active = false;
    for (int m = 0; m < M; ++m) {
      if (!br.active[m]) continue;
      energy[m] = hstats[2 * m] + enuc[m];
      const int nm = br.n[m];
      const double rms = std::sqrt(hstats[2 * m + 1] / ((double)nm * nm));
      iters[m] = step + 1;
      const bool handover = o->final_fp64 && precision == GBHF_PREC_MIXED;   // as scf.cu
      const double ce = handover ? std::max(o->conv_energy, 1e-9) : o->conv_energy;
      const double cd = handover ? std::max(o->conv_density, 1e-7) : o->conv_density;
      if (have_prev[m] && std::fabs(energy[m] - e_prev[m]) < ce && rms < cd) {
        conv[m] = 1;
        act[m] = 0;
      }
      e_prev[m] = energy[m];
      have_prev[m] = 1;
    }
    // converged molecules keep F(D) of their last step for the gradient
    GBHF_CUDA(c, cudaMemcpyAsync(Ffin, F, nst * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(D, Dn, nst * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    for (int m = 0; m < M; ++m) any_active |= act[m] != 0;
    c->prof.ph_other += ms_since(t_phase);
    c->prof.batch_steps = step + 1;
    if (!any_active && !o->final_fp64) break;
    if (!any_active) {
      if (precision == GBHF_PREC_MIXED && o->final_fp64) {
        // FP64 final iterations for every molecule (exact-mode rule of scf.cu)
        precision = GBHF_PREC_FP64;
        fp64_final_phase = true;
        std::fill(act.begin(), act.end(), 1);
        std::fill(conv.begin(), conv.end(), 0);
        std::fill(have_prev.begin(), have_prev.end(), 0);
        GBHF_TRY(br.set_active(act));
        continue;
      }
      break;
    }
    if (act != br.active) {
      GBHF_TRY(br.set_active(act));
      c->tasks.thr_all = -1;
    }
  }
  c->mol_active = nullptr;
  if (status != GBHF_OK) return status;
  for (int m = 0; m < M; ++m) {
    energies[m] = energy[m];
    if (iterations) iterations[m] = iters[m];
    if (converged_out) converged_out[m] = conv[m];
  }
  t_phase = clk::now();
  if (grads) {
    // D and W from the orbitals of the last F(D): D' = projector of F, W = D' F D' / 2
    std::vector<int> all(M, 1);
    GBHF_TRY(br.set_active(all));
    GBHF_TRY(b_density(br, Ffin, X, Dg, T1, Fp, P, P2, P3, d_g, d_coef));
    GBHF_TRY(br.gemm(false, false, 1.0, Dg, Ffin, 0.0, T1));
    GBHF_TRY(br.gemm(false, false, 0.5, T1, Dg, 0.0, Wm, true));
    DBuf<double> dgrad;
    GBHF_CUDA(c, dgrad.alloc(3 * (size_t)b.natoms));
    const double gs = o->schwarz_cutoff > 0 ? o->schwarz_cutoff : 1e-12;
    const double gm = o->grad_mixed_cutoff > 0 ? o->grad_mixed_cutoff : o->mixed_cutoff;
    if (o->autotune && !c->tuned[1]) GBHF_TRY(autotune_dev(c, 1, Dg, o->precision, gs, gm, 2, nullptr));
    GBHF_TRY(gradient_dev(c, Dg, Wm, gs, gm, o->precision, dgrad.p));
    GBHF_CUDA(c, cudaMemcpyAsync(grads, dgrad.p, 3 * (size_t)b.natoms * sizeof(double), cudaMemcpyDeviceToHost,
                                 c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->prof.ph_grad += ms_since(t_phase);
  for (int m = 0; m < M; ++m)
    if (!conv[m]) return fail(c, GBHF_ERR_NOT_CONVERGED, "molecule " + std::to_string(m) + ": SCF maxium steps exceeded");
  return GBHF_OK;
}

}  // namespace gbhf
