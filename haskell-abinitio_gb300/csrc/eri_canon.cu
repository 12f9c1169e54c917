// One-electron matrices, canonical ERI array, Fock from stored ERIs, Boys
// values and shell-pair Schwarz bounds (FP64, generic angular momentum).
#include <cmath>
#include <vector>

#include <algorithm>

#include "gbhf_internal.h"
#include "gbhf_md.cuh"

namespace gbhf {

__device__ __forceinline__ long tri_l(long n) { return n * (n + 1) / 2; }
__device__ __forceinline__ long flat2_dev(long dim, long x, long y) {
  if (x > y) {
    long t = x;
    x = y;
    y = t;
  }
  return x * dim - tri_l(x - 1) + (y - x);
}

// ------------------------------------------------------------ Boys ----
__global__ void k_boys(bool ref, const double* __restrict__ grid, const double* __restrict__ tab, int mmax, int n,
                       const double* __restrict__ x, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double F[MD_LMAX + 12];
  boys_generic(ref, grid, tab, mmax, x[i], F);
  for (int m = 0; m <= mmax; ++m) out[i * (mmax + 1) + m] = F[m];
}

gbhf_status boys_dev(gbhf_ctx* c, bool ref, int mmax, int n, const double* d_x, double* d_out) {
  if (mmax < 0 || mmax > MD_LMAX + 8 || (!ref && mmax + BOYS64_NTERM > BOYS_NCOL) || (ref && mmax > 9))
    return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_boys: m_max out of range");
  if (n <= 0) return GBHF_OK;
  k_boys<<<(n + 127) / 128, 128, 0, c->stream>>>(ref, c->boys_ref.p, c->boys64.p, mmax, n, d_x, d_out);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// ------------------------------------------------- one-electron terms ----
// obaraSaika table s(m,n), m <= 2, n <= 4 (Integrals/IntegralsEvaluation.hs:209-221)
__device__ inline void os_table(double gamma, double s00, double pax, double pbx, int M, int N, double s[3][5]) {
  const double c = 1.0 / (2.0 * gamma);
  for (int m = 0; m <= M; ++m)
    for (int n = 0; n <= N; ++n) {
      double v;
      if (m == 0 && n == 0) {
        v = s00;
      } else if (m == 0) {
        v = pbx * s[0][n - 1] + (n >= 2 ? c * (n - 1) * s[0][n - 2] : 0.0);
      } else if (n == 0) {
        v = pax * s[m - 1][0] + (m >= 2 ? c * (m - 1) * s[m - 2][0] : 0.0);
      } else {
        v = pax * s[m - 1][n] + c * ((m >= 2 ? (m - 1) * s[m - 2][n] : 0.0) + n * s[m - 1][n - 1]);
      }
      s[m][n] = v;
    }
}

// Row i (global function) pairs with the functions j >= i of its molecule;
// nuclear attraction over that molecule's atoms.  Output: the flat upper
// triangle of one molecule (moff == nullptr), or both triangles of the
// molecule's block of stacked square matrices.
__global__ void k_onee(bool ref, int nbf, const int* __restrict__ fmol, const int* __restrict__ mfo,
                       const int* __restrict__ mao, const long long* __restrict__ moff, const double* __restrict__ xyz,
                       const double* __restrict__ Z, const int* __restrict__ fn, const double* __restrict__ coef,
                       const double* __restrict__ expo, const double* __restrict__ grid,
                       const double* __restrict__ tab, double* __restrict__ S, double* __restrict__ H) {
  const int i = blockIdx.y;
  const int mol = fmol[i];
  const int f0m = mfo[mol], nm = mfo[mol + 1] - f0m, a0 = mao[mol], a1 = mao[mol + 1];
  const int il = i - f0m, jl = blockIdx.x * blockDim.x + threadIdx.x;
  if (jl >= nm || jl < il) return;
  const int j = f0m + jl;
  const DevFn f = load_fn(fn, i), g = load_fn(fn, j);
  const double *A = xyz + 3 * f.atom, *B = xyz + 3 * g.atom;
  const long out = moff ? (long)(moff[mol] + (long long)il * nm + jl) : flat2_dev(nbf, i, j);
  const long out_t = moff ? (long)(moff[mol] + (long long)jl * nm + il) : out;
  // overlap (sijContracted, IntegralsEvaluation.hs:181-206)
  bool same = false;
  if (ref) {
    same = f.l[0] == g.l[0] && f.l[1] == g.l[1] && f.l[2] == g.l[2] && f.np == g.np && A[0] == B[0] &&
           A[1] == B[1] && A[2] == B[2];
    for (int k = 0; same && k < f.np; ++k)
      same = coef[f.off + k] == coef[g.off + k] && expo[f.off + k] == expo[g.off + k];
  }
  double s_sum = 0, t_sum = 0, v_sum = 0;
  const int L = f.l[0] + f.l[1] + f.l[2] + g.l[0] + g.l[1] + g.l[2];
  double F[MD_LMAX + 1];
  double R[MD_D * MD_D * MD_D];
  for (int p1 = 0; p1 < f.np; ++p1)
    for (int p2 = 0; p2 < g.np; ++p2) {
      const double c1 = coef[f.off + p1], e1 = expo[f.off + p1];
      const double c2 = coef[g.off + p2], e2 = expo[g.off + p2];
      const double p = e1 + e2, mu = e1 * e2 / p;
      const double cte = sqrt(GBHF_PI / p);
      double P[3], sx[3], tx[3];
      EAx E[3];
      for (int x = 0; x < 3; ++x) {
        P[x] = (e1 * A[x] + e2 * B[x]) / p;
        const double ab = A[x] - B[x];
        const double ex = exp(-mu * ab * ab);
        double s[3][5];
        const int l1 = f.l[x], l2 = g.l[x];
        os_table(p, ex * cte, P[x] - A[x], P[x] - B[x], l1, l2 + 2, s);
        sx[x] = s[l1][l2];
        // kinetic 1-D term (tab, IntegralsEvaluation.hs:263-280)
        tx[x] = -2.0 * e2 * e2 * s[l1][l2 + 2] + e2 * (2 * l2 + 1) * s[l1][l2] -
                (l2 >= 2 ? 0.5 * l2 * (l2 - 1) * s[l1][l2 - 2] : 0.0);
        e_axis(E[x], l1, l2, p, P[x] - A[x], P[x] - B[x], ex);
      }
      s_sum += (c1 * c2) * (sx[0] * sx[1] * sx[2]);
      t_sum += c1 * c2 * (tx[0] * sx[1] * sx[2] + sx[0] * tx[1] * sx[2] + sx[0] * sx[1] * tx[2]);
      // nuclear attraction (vijHermite/mcMurchie, IntegralsEvaluation.hs:395-414)
      for (int cn = a0; cn < a1; ++cn) {
        const double* Cc = xyz + 3 * cn;
        const double PC[3] = {P[0] - Cc[0], P[1] - Cc[1], P[2] - Cc[2]};
        boys_generic(ref, grid, tab, L, p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]), F);
        hermite_r<MD_LMAX>(L, p, PC[0], PC[1], PC[2], F, R);
        double sum = 0;
        for (int t = 0; t <= f.l[0] + g.l[0]; ++t)
          for (int u = 0; u <= f.l[1] + g.l[1]; ++u)
            for (int v = 0; v <= f.l[2] + g.l[2]; ++v)
              sum += E[0].get(f.l[0], g.l[0], t) * E[1].get(f.l[1], g.l[1], u) * E[2].get(f.l[2], g.l[2], v) *
                     R[(t * MD_D + u) * MD_D + v];
        v_sum += (-Z[cn]) * (c1 * c2 * 2.0 * (GBHF_PI / p) * sum);
      }
    }
  const double sv = same ? 1.0 : s_sum, hv = t_sum + v_sum;
  if (S) S[out] = sv;
  if (H) H[out] = hv;
  if (moff) {
    if (S) S[out_t] = sv;
    if (H) H[out_t] = hv;
  }
}

// Exact mode with complete shells: one warp per shell pair (A, B) of a
// molecule, l_A >= l_B, every component pair at once.  The primitive pairs'
// Obara-Saika tables (overlap, kinetic) and Hermite E coefficients serve all
// NA x NB components, and the nuclear-attraction R^n_tuv of one (primitive
// pair, atom) all of them too; lanes take primitive pairs, and when a pair has
// fewer primitive pairs than lanes, slices of the molecule's atoms as well.
// Component integrals use the first component's contraction coefficients
// times the shells' component ratios (d shells).  Same formulas as k_onee.
__host__ __device__ constexpr int cart_l(int L, int k, int axis) {
  // components in createCGF order: x, y, z; xx, xy, xz, yy, yz, zz
  return L == 0 ? 0
         : L == 1 ? (k == axis ? 1 : 0)
                  : (axis == 0 ? (k == 0 ? 2 : (k == 1 || k == 2) ? 1 : 0)
                     : axis == 1 ? (k == 3 ? 2 : (k == 1 || k == 4) ? 1 : 0)
                                 : (k == 5 ? 2 : (k == 2 || k == 4) ? 1 : 0));
}

struct OneeArgs {
  const int2* pairs;
  int npairs;
  int nbf;
  const int *f0, *smol, *mfo, *mao, *mn, *fn;
  const long long* moff;   // stacked output (nullptr: flat upper triangle of one molecule)
  const double *xyz, *Z, *coef, *expo, *tab, *sscale;
  double *S, *H;
};

constexpr int ONEE_WARPS = 4;

template <int N>
__device__ __forceinline__ void warp_sum_all(double (&v)[N]) {
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
}

template <int LA, int LB>
__global__ void __launch_bounds__(ONEE_WARPS * 32) k_onee_sh(OneeArgs a) {
  constexpr int NA = ncart_c(LA), NB = ncart_c(LB), NAB = NA * NB, L = LA + LB;
  const int w = blockIdx.x * ONEE_WARPS + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= a.npairs) return;   // whole warps
  const int2 pr = a.pairs[w];
  const int A = pr.x, B = pr.y;
  const int mol = a.smol[A];
  const int fa = a.mfo[mol] + a.f0[A], fb = a.mfo[mol] + a.f0[B];
  const DevFn f = load_fn(a.fn, fa), g = load_fn(a.fn, fb);
  const double* RA = a.xyz + 3 * f.atom;
  const double* RB = a.xyz + 3 * g.atom;
  const int kb = f.np * g.np;
  double sv[NAB], tv[NAB], vv[NAB];
#pragma unroll
  for (int i = 0; i < NAB; ++i) sv[i] = tv[i] = vv[i] = 0.0;
  // overlap and kinetic (sijContracted / tijContracted, IntegralsEvaluation.hs:181-206, 252-280)
  for (int kp = lane; kp < kb; kp += 32) {
    const int p1 = kp / g.np, p2 = kp - p1 * g.np;
    const double c1 = a.coef[f.off + p1], e1 = a.expo[f.off + p1];
    const double c2 = a.coef[g.off + p2], e2 = a.expo[g.off + p2];
    const double p = e1 + e2, mu = e1 * e2 / p, cte = sqrt(GBHF_PI / p);
    double sx[3][LA + 1][LB + 1], tx[3][LA + 1][LB + 1];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      const double P = (e1 * RA[x] + e2 * RB[x]) / p, ab = RA[x] - RB[x];
      double st[3][5];
      os_table(p, exp(-mu * ab * ab) * cte, P - RA[x], P - RB[x], LA, LB + 2, st);
#pragma unroll
      for (int i = 0; i <= LA; ++i)
#pragma unroll
        for (int j = 0; j <= LB; ++j) {
          sx[x][i][j] = st[i][j];
          tx[x][i][j] = -2.0 * e2 * e2 * st[i][j + 2] + e2 * (2 * j + 1) * st[i][j] -
                        (j >= 2 ? 0.5 * j * (j - 1) * st[i][j - 2] : 0.0);
        }
    }
    const double cc = c1 * c2;
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
      for (int ib = 0; ib < NB; ++ib) {
        const int ax = cart_l(LA, ia, 0), ay = cart_l(LA, ia, 1), az = cart_l(LA, ia, 2);
        const int bx = cart_l(LB, ib, 0), by = cart_l(LB, ib, 1), bz = cart_l(LB, ib, 2);
        const double X = sx[0][ax][bx], Y = sx[1][ay][by], Zs = sx[2][az][bz];
        sv[ia * NB + ib] += cc * (X * Y * Zs);
        tv[ia * NB + ib] += cc * (tx[0][ax][bx] * Y * Zs + X * tx[1][ay][by] * Zs + X * Y * tx[2][az][bz]);
      }
  }
  // nuclear attraction (vijHermite/mcMurchie, IntegralsEvaluation.hs:395-414)
  const int at0 = a.mao[mol], nat = a.mao[mol + 1] - at0;
  if (a.H && kb > 0) {
    const int nch = max(1, min(nat, 32 / kb));
    const int cs = (nat + nch - 1) / nch;
    for (int it = lane; it < kb * nch; it += 32) {
      const int kp = it / nch, ch = it - kp * nch;
      const int p1 = kp / g.np, p2 = kp - p1 * g.np;
      const double c1 = a.coef[f.off + p1], e1 = a.expo[f.off + p1];
      const double c2 = a.coef[g.off + p2], e2 = a.expo[g.off + p2];
      const double p = e1 + e2, mu = e1 * e2 / p;
      double P[3];
      EAx E[3];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        P[x] = (e1 * RA[x] + e2 * RB[x]) / p;
        const double ab = RA[x] - RB[x];
        e_axis(E[x], LA, LB, p, P[x] - RA[x], P[x] - RB[x], exp(-mu * ab * ab));
      }
      const double pref = c1 * c2 * 2.0 * (GBHF_PI / p);
      const int c_end = min(nat, (ch + 1) * cs);
      for (int cn = at0 + ch * cs; cn < at0 + c_end; ++cn) {
        const double* Cc = a.xyz + 3 * cn;
        const double PC[3] = {P[0] - Cc[0], P[1] - Cc[1], P[2] - Cc[2]};
        double F[L + 1];
        constexpr int D = L + 1;
        double R[D * D * D];
        boys_generic(false, nullptr, a.tab, L, p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]), F);
        hermite_r<L>(L, p, PC[0], PC[1], PC[2], F, R);
        const double zp = -a.Z[cn] * pref;
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
          for (int ib = 0; ib < NB; ++ib) {
            const int ax = cart_l(LA, ia, 0), ay = cart_l(LA, ia, 1), az = cart_l(LA, ia, 2);
            const int bx = cart_l(LB, ib, 0), by = cart_l(LB, ib, 1), bz = cart_l(LB, ib, 2);
            double sum = 0;
#pragma unroll
            for (int t = 0; t <= ax + bx; ++t)
#pragma unroll
              for (int u = 0; u <= ay + by; ++u)
#pragma unroll
                for (int v = 0; v <= az + bz; ++v)
                  sum += E[0].get(ax, bx, t) * E[1].get(ay, by, u) * E[2].get(az, bz, v) * R[(t * D + u) * D + v];
            vv[ia * NB + ib] += zp * sum;
          }
      }
    }
  }
  warp_sum_all(sv);
  warp_sum_all(tv);
  warp_sum_all(vv);
  const int nm = a.mn[mol];
#pragma unroll
  for (int ia = 0; ia < NA; ++ia)
#pragma unroll
    for (int ib = 0; ib < NB; ++ib) {
      const int k = ia * NB + ib;
      if ((k & 31) != lane || (A == B && ia > ib)) continue;
      const double sc = a.sscale[6 * A + ia] * a.sscale[6 * B + ib];
      const double s_ = sc * sv[k], h_ = sc * (tv[k] + vv[k]);
      const int li = a.f0[A] + ia, lj = a.f0[B] + ib;
      if (a.moff) {
        const long long o1 = a.moff[mol] + (long long)li * nm + lj, o2 = a.moff[mol] + (long long)lj * nm + li;
        if (a.S) a.S[o1] = s_, a.S[o2] = s_;
        if (a.H) a.H[o1] = h_, a.H[o2] = h_;
      } else {
        const long o = flat2_dev(a.nbf, fa + ia, fb + ib);
        if (a.S) a.S[o] = s_;
        if (a.H) a.H[o] = h_;
      }
    }
}

// Shell pairs (A, B), l_A >= l_B, of each molecule, grouped by pair class.
static gbhf_status onee_pair_lists(gbhf_ctx* c) {
  if (c->onee_gen == c->basis_gen) return GBHF_OK;
  const Basis& b = c->basis;
  std::vector<int2> lst[NPCLS];
  const int ns = (int)b.shells.size();
  std::vector<std::vector<int>> by_mol(b.nmol);
  for (int A = 0; A < ns; ++A) by_mol[b.shells[A].mol].push_back(A);
  for (const auto& sh : by_mol)
    for (size_t ia = 0; ia < sh.size(); ++ia)
      for (size_t ib = 0; ib <= ia; ++ib) {
        int x = sh[ia], y = sh[ib];
        if (b.shells[y].L > b.shells[x].L) std::swap(x, y);
        lst[pair_class_of(b.shells[x].L, b.shells[y].L)].push_back(make_int2(x, y));
      }
  std::vector<int2> all;
  c->onee_cls[0] = 0;
  for (int k = 0; k < NPCLS; ++k) {
    all.insert(all.end(), lst[k].begin(), lst[k].end());
    c->onee_cls[k + 1] = (int)all.size();
  }
  GBHF_CUDA(c, c->onee_pairs.alloc(std::max<size_t>(all.size(), 1)));
  if (!all.empty())
    GBHF_CUDA(c, cudaMemcpyAsync(c->onee_pairs.p, all.data(), all.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                 c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));   // `all` goes out of scope
  c->onee_gen = c->basis_gen;
  return GBHF_OK;
}

template <int LA, int LB>
static void onee_sh_class(gbhf_ctx* c, OneeArgs a, int k) {
  a.pairs = c->onee_pairs.p + c->onee_cls[k];
  a.npairs = c->onee_cls[k + 1] - c->onee_cls[k];
  if (a.npairs <= 0) return;
  k_onee_sh<LA, LB><<<(a.npairs + ONEE_WARPS - 1) / ONEE_WARPS, ONEE_WARPS * 32, 0, c->stream>>>(a);
  count_launch(c);
}

static gbhf_status onee_launch(gbhf_ctx* c, bool ref, bool stacked, double* d_S, double* d_H) {
  const Basis& b = c->basis;
  if (b.maxL > 2) return fail(c, GBHF_ERR_UNSUPPORTED, "one-electron integrals support s, p, d functions");
  if (ref && !c->have_grid) return fail(c, GBHF_ERR_BAD_INPUT, "reference mode needs gbhf_set_boys_grid");
  if (!stacked && b.nmol != 1) return fail(c, GBHF_ERR_BAD_INPUT, "flat one-electron matrices need one molecule");
  GBHF_TRY(ensure_shell_arrays(c));
  const TaskLists& t = c->tasks;
  if (!ref && b.shells_ok) {
    GBHF_TRY(onee_pair_lists(c));
    OneeArgs a;
    a.nbf = b.nbf;
    a.f0 = t.f0.p;
    a.smol = t.smol.p;
    a.mfo = t.mfo.p;
    a.mao = t.mao.p;
    a.mn = t.mn.p;
    a.fn = c->d_fn.p;
    a.moff = stacked ? t.moff.p : nullptr;
    a.xyz = c->d_xyz.p;
    a.Z = c->d_Z.p;
    a.coef = c->d_coef.p;
    a.expo = c->d_exp.p;
    a.tab = c->boys64.p;
    a.sscale = t.sscale.p;
    a.S = d_S;
    a.H = d_H;
    onee_sh_class<0, 0>(c, a, 0);
    onee_sh_class<1, 0>(c, a, 1);
    onee_sh_class<1, 1>(c, a, 2);
    onee_sh_class<2, 0>(c, a, 3);
    onee_sh_class<2, 1>(c, a, 4);
    onee_sh_class<2, 2>(c, a, 5);
    GBHF_CUDA(c, cudaGetLastError());
    return GBHF_OK;
  }
  int max_fn = 0;
  for (int m = 0; m < b.nmol; ++m) max_fn = std::max(max_fn, b.mol_fn_off[m + 1] - b.mol_fn_off[m]);
  dim3 grid((max_fn + 63) / 64, b.nbf);
  k_onee<<<grid, 64, 0, c->stream>>>(ref, b.nbf, t.fmol.p, t.mfo.p, t.mao.p, stacked ? t.moff.p : nullptr,
                                      c->d_xyz.p, c->d_Z.p, c->d_fn.p, c->d_coef.p, c->d_exp.p, c->boys_ref.p,
                                      c->boys64.p, d_S, d_H);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

gbhf_status onee_matrices(gbhf_ctx* c, bool ref, double* d_S, double* d_H) {
  return onee_launch(c, ref, false, d_S, d_H);
}

gbhf_status onee_stacked(gbhf_ctx* c, double* d_S, double* d_H) { return onee_launch(c, false, true, d_S, d_H); }

// ------------------------------------------------- canonical ERIs ----
// Key (i<=j | k<=l) with (i,j) <= (k,l) lexicographically <=> flat pair
// indices P = flat(i,j) <= Q = flat(k,l).  The position in the reference's
// enumeration order (calcIntegrals, HartreeFock.hs:166-181) is
// off[i*n+j] + (k == i ? l - j : (n - j) + sum_{k'=i+1}^{k-1}(n-k') + l - k).
__device__ __forceinline__ long canon_pos(const long* __restrict__ off, long n, long i, long j, long k, long l) {
  long idx = off[i * n + j];
  if (k == i) return idx + (l - j);
  idx += n - j;
  const long m = k - i - 1;
  idx += m * n - (m * i + tri_l(m));
  return idx + (l - k);
}

__device__ __forceinline__ void sort_key(long& i, long& j, long& k, long& l) {
  long t;
  if (i > j) { t = i; i = j; j = t; }
  if (k > l) { t = k; k = l; l = t; }
  if (i > k || (i == k && j > l)) {
    t = i; i = k; k = t;
    t = j; j = l; l = t;
  }
}

template <int LM>
__global__ void k_eri_canonical(bool ref, int nbf, const int* __restrict__ pair_i, const int* __restrict__ pair_j,
                                long npair, const long* __restrict__ off, const double* __restrict__ xyz,
                                const int* __restrict__ fn, const double* __restrict__ coef,
                                const double* __restrict__ expo, const double* __restrict__ grid,
                                const double* __restrict__ tab, double* __restrict__ eri) {
  const long P = blockIdx.y;
  const long Q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (Q >= npair || Q < P) return;
  const long i = pair_i[P], j = pair_j[P], k = pair_i[Q], l = pair_j[Q];
  eri[canon_pos(off, nbf, i, j, k, l)] =
      eri_fn_generic<LM>(ref, xyz, fn, coef, expo, grid, tab, (int)i, (int)j, (int)k, (int)l);
}

// The same array with a warp per (P <= Q): the lanes take the quartet's
// primitive quartets in turn and a shuffle sum closes it (the atoms of the SAD
// guess have up to 6^4 primitive quartets per function quartet).
template <int LM>
__global__ void k_eri_canonical_warp(bool ref, int nbf, const int* __restrict__ pair_i,
                                     const int* __restrict__ pair_j, long npair, const long* __restrict__ off,
                                     const double* __restrict__ xyz, const int* __restrict__ fn,
                                     const double* __restrict__ coef, const double* __restrict__ expo,
                                     const double* __restrict__ grid, const double* __restrict__ tab,
                                     double* __restrict__ eri) {
  const long P = blockIdx.y;
  const long Q = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (Q >= npair || Q < P) return;   // whole warps leave together
  const long i = pair_i[P], j = pair_j[P], k = pair_i[Q], l = pair_j[Q];
  double v = eri_fn_generic<LM>(ref, xyz, fn, coef, expo, grid, tab, (int)i, (int)j, (int)k, (int)l, lane, 32);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) eri[canon_pos(off, nbf, i, j, k, l)] = v;
}

static void canonical_offsets(long n, std::vector<long>& off) {
  off.assign(n * n, 0);
  long acc = 0;
  for (long i = 0; i < n; ++i)
    for (long j = i; j < n; ++j) {
      off[i * n + j] = acc;
      acc += (n - j) + (n - i - 1) * (n - i) / 2;
    }
}

struct CanonAux {
  DBuf<int> pi, pj;
  DBuf<long> off;
};

static gbhf_status canon_aux(gbhf_ctx* c, CanonAux& aux) {
  const long n = c->basis.nbf, np = n * (n + 1) / 2;
  std::vector<int> hi(np), hj(np);
  long q = 0;
  for (long i = 0; i < n; ++i)
    for (long j = i; j < n; ++j, ++q) {
      hi[q] = (int)i;
      hj[q] = (int)j;
    }
  std::vector<long> off;
  canonical_offsets(n, off);
  GBHF_CUDA(c, aux.pi.alloc(np));
  GBHF_CUDA(c, aux.pj.alloc(np));
  GBHF_CUDA(c, aux.off.alloc(n * n));
  GBHF_CUDA(c, cudaMemcpyAsync(aux.pi.p, hi.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(aux.pj.p, hj.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(aux.off.p, off.data(), n * n * sizeof(long), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

gbhf_status eri_canonical_dev(gbhf_ctx* c, bool ref, double* d_eri) {
  const Basis& b = c->basis;
  if (b.maxL > 2) return fail(c, GBHF_ERR_UNSUPPORTED, "canonical ERIs support s, p and d functions");
  if (ref && !c->have_grid) return fail(c, GBHF_ERR_BAD_INPUT, "reference mode needs gbhf_set_boys_grid");
  CanonAux aux;
  GBHF_TRY(canon_aux(c, aux));
  const long np = (long)b.nbf * (b.nbf + 1) / 2;
  if (np > 65535) return fail(c, GBHF_ERR_UNSUPPORTED, "canonical ERI array too large");
  dim3 grid((unsigned)((np + 127) / 128), (unsigned)np);
  // per-thread Hermite cubes sized for the largest total angular momentum: s/p quartets L <= 4, d L <= 8
  if (!ref) {   // exact numerics: a warp per quartet (the reference mode keeps its serial primitive order)
    dim3 wgrid((unsigned)((np + 3) / 4), (unsigned)np);
    if (b.maxL <= 1)
      k_eri_canonical_warp<MD_LMAX><<<wgrid, 128, 0, c->stream>>>(ref, b.nbf, aux.pi.p, aux.pj.p, np, aux.off.p,
                                                                  c->d_xyz.p, c->d_fn.p, c->d_coef.p, c->d_exp.p,
                                                                  c->boys_ref.p, c->boys64.p, d_eri);
    else
      k_eri_canonical_warp<8><<<wgrid, 128, 0, c->stream>>>(ref, b.nbf, aux.pi.p, aux.pj.p, np, aux.off.p,
                                                            c->d_xyz.p, c->d_fn.p, c->d_coef.p, c->d_exp.p,
                                                            c->boys_ref.p, c->boys64.p, d_eri);
  } else if (b.maxL <= 1)
    k_eri_canonical<MD_LMAX><<<grid, 128, 0, c->stream>>>(ref, b.nbf, aux.pi.p, aux.pj.p, np, aux.off.p, c->d_xyz.p,
                                                          c->d_fn.p, c->d_coef.p, c->d_exp.p, c->boys_ref.p,
                                                          c->boys64.p, d_eri);
  else
    k_eri_canonical<8><<<grid, 128, 0, c->stream>>>(ref, b.nbf, aux.pi.p, aux.pj.p, np, aux.off.p, c->d_xyz.p,
                                                    c->d_fn.p, c->d_coef.p, c->d_exp.p, c->boys_ref.p, c->boys64.p,
                                                    d_eri);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

// calcGmatrix/sliceIntegrals (HartreeFock.hs:225-260):
// F_ab = H_ab + sum_l sum_k D_lk [(ab|kl) - 1/2 (al|kb)], flat in and out.
__global__ void k_fock_canonical(int n, const long* __restrict__ off, const double* __restrict__ H,
                                 const double* __restrict__ D, const double* __restrict__ eri,
                                 double* __restrict__ F) {
  const int a = blockIdx.y;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n || b < a) return;
  double g = 0;
  for (long l = 0; l < n; ++l) {
    double row = 0;
    for (long k = 0; k < n; ++k) {
      long i1 = a, j1 = b, k1 = k, l1 = l;
      sort_key(i1, j1, k1, l1);
      long i2 = a, j2 = l, k2 = k, l2 = b;
      sort_key(i2, j2, k2, l2);
      const double coul = eri[canon_pos(off, n, i1, j1, k1, l1)];
      const double exch = eri[canon_pos(off, n, i2, j2, k2, l2)];
      row += D[flat2_dev(n, l, k)] * (coul - 0.5 * exch);
    }
    g += row;
  }
  const long o = flat2_dev(n, a, b);
  F[o] = H[o] + g;
}

gbhf_status fock_canonical_dev(gbhf_ctx* c, const double* d_H, const double* d_D, const double* d_eri, double* d_F) {
  CanonAux aux;
  GBHF_TRY(canon_aux(c, aux));
  const int n = c->basis.nbf;
  dim3 grid((n + 63) / 64, n);
  k_fock_canonical<<<grid, 64, 0, c->stream>>>(n, aux.off.p, d_H, d_D, d_eri, d_F);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}


}  // namespace gbhf

namespace gbhf {

// generateGridBoys 0.1 (NumericalTools/TableBoys.hs:58-63) on the device:
// grid[m*1001+i] = boysF m (0.1 i).  boysF (Boys.hs:54-66): m = 0 from erf
// (asymptotic beyond 50); m >= 1 by Kummer's integral with the 256-point
// Gauss-Legendre rule that kummer selects for err = 0.1 (Boys.hs:106-118).
__global__ void k_boys_ref_grid(const double* __restrict__ xq, const double* __restrict__ wq, int nq,
                                double* __restrict__ grid) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 15 * 1001) return;
  const int m = idx / 1001, i = idx % 1001;
  const double x = 0.1 * i;
  double v;
  if (m == 0) {
    if (x > 50) v = asympt_boys_ref(0.0, x);
    else if (x > 0.0) v = 0.5 * sqrt(GBHF_PI / x) * erf(sqrt(x));
    else v = 1.0;
  } else {
    const double n = m, a = n + 0.5, b = n + 1.5, z = -x;
    const double gamma_factor = tgamma(b) / (tgamma(a) * tgamma(b - a));
    const double e = exp(1.0);
    double acc = 0;
    for (int k = 0; k < nq; ++k) {
      const double t1 = 0.5 * ((1.0 - 0.0) * xq[k] + 1.0 + 0.0);
      const double t2 = 0.5 * ((1.0 - 0.0) * (-xq[k]) + 1.0 + 0.0);
      const double f1 = (pow(e, z * t1) * pow(1 - t1, b - a - 1)) * pow(t1, a - 1);
      const double f2 = (pow(e, z * t2) * pow(1 - t2, b - a - 1)) * pow(t2, a - 1);
      acc += wq[k] * (f1 + f2);
    }
    v = gamma_factor * (0.5 * (1.0 - 0.0) * acc) / (2 * n + 1);
  }
  grid[idx] = v;
}

// Positive Gauss-Legendre nodes/weights of the n-point rule, ascending
// (Newton iteration on P_n in long double).
static void gauss_legendre_pos(int n, std::vector<double>& xs, std::vector<double>& ws) {
  const int half = n / 2;
  xs.assign(half, 0.0);
  ws.assign(half, 0.0);
  for (int i = 0; i < half; ++i) {
    long double z = cosl(3.14159265358979323846264338327950288L * (i + 0.75L) / (n + 0.5L));
    long double pp = 1;
    for (int it = 0; it < 100; ++it) {
      long double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        const long double p3 = p2;
        p2 = p1;
        p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      const long double z1 = z;
      z = z1 - p1 / pp;
      if (fabsl(z - z1) < 1e-30L) break;
    }
    long double p1 = 1, p2 = 0;
    for (int j = 1; j <= n; ++j) {
      const long double p3 = p2;
      p2 = p1;
      p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
    }
    pp = n * (z * p1 - p2) / (z * z - 1);
    xs[half - 1 - i] = (double)z;
    ws[half - 1 - i] = (double)(2.0L / ((1 - z * z) * pp * pp));
  }
}

gbhf_status boys_ref_grid_dev(gbhf_ctx* c, double* d_grid) {
  std::vector<double> xs, wsv;
  gauss_legendre_pos(256, xs, wsv);
  DBuf<double> dx, dw;
  GBHF_CUDA(c, dx.alloc(xs.size()));
  GBHF_CUDA(c, dw.alloc(wsv.size()));
  GBHF_CUDA(c, cudaMemcpyAsync(dx.p, xs.data(), xs.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dw.p, wsv.data(), wsv.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  k_boys_ref_grid<<<(15 * 1001 + 127) / 128, 128, 0, c->stream>>>(dx.p, dw.p, (int)xs.size(), d_grid);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

}  // namespace gbhf
