// Direct J/K build and Schwarz bounds for the quartet classes that hold a d
// shell: one warp per contracted shell quartet (mdwarp.cuh).
//
// The task lists, unique-quartet rule, degeneracy weights and scatter are
// those of the s/p kernels (k_jk): a task is (bra pair, up to 32 kets of one
// segment, a range of bra primitives); here the warp walks the task's kets
// one after another and, for each, sums the primitive quartets into the
// lane-owned entries of the (ab|cd) block before the J and K scatter.
#include <algorithm>

#include "gbhf_internal.h"
#include "mdwarp.cuh"

namespace gbhf {

constexpr int JKD_WARPS = 2;
constexpr int JKD_THREADS = 32 * JKD_WARPS;
constexpr int TUV_BYTES = ((nherm(BOYSH_LMAX) * 4 + 15) / 16) * 16;

template <typename T>
struct JKDArgs {
  const int4* tasks;
  const int* range;   // [start, end)
  int* counter;
  const int* pA;
  const int* pB;
  const int* poff;
  const int* kseg;
  const int4* seg;
  const T* bra;
  const T* ket;
  long long npp;
  const int* shell_f0;
  const int* pmol;
  const int* mn;
  const long long* moff;
  const double* sscale;   // per shell 6 component scales (1 for s and p)
  const T* D;
  double* G;
  const T* boys;
  unsigned long long* stats;
  int with_j;             // 0: exchange only
  const double* Q;        // Schwarz bound of each pair
  double thr;             // per-quartet screening on the six density blocks (as k_jk)
};

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(JKD_THREADS) k_jkd(JKDArgs<T> a) {
  using C = MDCfg<LA, LB, LC, LD, 0>;
  extern __shared__ __align__(16) unsigned char jkd_smem[];
  int* tuv = reinterpret_cast<int*>(jkd_smem);
  md_fill_tuv(tuv, C::L);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* ws = reinterpret_cast<T*>(jkd_smem + TUV_BYTES) + warp * C::WS;
  T* sbra = ws + C::OFF_SB;
  T* I = ws + C::OFF_R;   // contracted block for the scatter (R is free by then)
  const int start = a.range[0], ntask = a.range[1] - start;
  const long long npp = a.npp;
  unsigned long long cnt_q = 0, cnt_p = 0;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(a.counter, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntask) break;
    const int4 task = a.tasks[start + t];
    const int ib = task.x;
    const int mol = a.pmol[ib];
    const int n = a.mn[mol];
    const T* __restrict__ Dm = a.D + a.moff[mol];
    double* __restrict__ Gm = a.G + a.moff[mol];
    const int kb0 = task.w & 0xffff, Kb = (task.w >> 16) - kb0, pb0 = a.poff[ib] + kb0;
    const unsigned rkb = (65536u + Kb - 1) / Kb;   // idx / Kb = (idx * rkb) >> 16 for idx < 16 * 36
    for (int idx = lane; idx < BRA_NJK * Kb; idx += 32) {
      const int f = (int)(((unsigned)idx * rkb) >> 16), k = idx - f * Kb;
      sbra[k * BRA_SB + f] = a.bra[(long long)f * npp + pb0 + k];
    }
    __syncwarp();
    const int A = a.pA[ib], B = a.pB[ib];
    const int a0 = a.shell_f0[A], b0 = a.shell_f0[B];
    for (int q = 0; q < task.z; ++q) {
      const int jk = task.y + q;
      const int Cs = a.pA[jk], Ds = a.pB[jk];
      const int c0 = a.shell_f0[Cs], d0 = a.shell_f0[Ds];
      {   // exact screening on the six density blocks of the quartet (as k_jk)
        double dmx = 0.0;
        constexpr int NB6 = C::NAB + C::NCD + (C::NA + C::NB) * (C::NC + C::ND);
        for (int e = lane; e < NB6; e += 32) {
          int r, q2;
          if (e < C::NAB) {
            r = a0 + e / C::NB;
            q2 = b0 + e % C::NB;
          } else if (e < C::NAB + C::NCD) {
            r = c0 + (e - C::NAB) / C::ND;
            q2 = d0 + (e - C::NAB) % C::ND;
          } else {
            const int f = e - C::NAB - C::NCD, rr = f / (C::NC + C::ND), cc = f % (C::NC + C::ND);
            r = rr < C::NA ? a0 + rr : b0 + (rr - C::NA);
            q2 = cc < C::NC ? c0 + cc : d0 + (cc - C::NC);
          }
          dmx = fmax(dmx, fabs((double)Dm[(long long)r * n + q2]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dmx = fmax(dmx, __shfl_xor_sync(0xffffffffu, dmx, o));
        if (a.Q[ib] * a.Q[jk] * dmx < a.thr) continue;   // warp-uniform
      }
      const int4 sg = a.seg[a.kseg[jk]];
      const int K = sg.z, len = sg.y - sg.x;
      const long long base = (long long)sg.w + (jk - sg.x);
      T acc[C::NPL];
#pragma unroll
      for (int k = 0; k < C::NPL; ++k) acc[k] = T(0);
      for (int kb = 0; kb < Kb; ++kb) {
        MDPrim<T> bp;
        md_row_prim(sbra + kb * BRA_SB, bp);
        md_bra_e<C>(ws, bp, lane);
        for (int kc = 0; kc < K; ++kc) {
          MDPrim<T> kp;
          md_load_prim(a.ket, npp, base + (long long)kc * len, kp);
          md_prim_x<C>(ws, tuv, bp, kp, a.boys, lane);
          md_bra_acc<C>(ws, acc, lane);
          __syncwarp();
        }
      }
      cnt_q += kb0 == 0;
      cnt_p += (unsigned long long)Kb * K;
      // ---- scatter into G'' (as k_jk), with the d-component scales
      const T s = (A == B ? T(0.5) : T(1)) * (Cs == Ds ? T(0.5) : T(1)) * (ib == jk ? T(0.5) : T(1));
#pragma unroll
      for (int k = 0; k < C::NPL; ++k) {
        const int e = lane + 32 * k;
        if (e < C::NOUT) {
          const int ab = e / C::NCD, cd = e - ab * C::NCD;
          const int ia = ab / C::NB, ibb = ab - ia * C::NB, ic = cd / C::ND, id = cd - ic * C::ND;
          const double sc = a.sscale[6 * A + ia] * a.sscale[6 * B + ibb] * a.sscale[6 * Cs + ic] * a.sscale[6 * Ds + id];
          I[e] = acc[k] * (s * T(sc));
        }
      }
      __syncwarp();
      for (int ab = lane; a.with_j && ab < C::NAB; ab += 32) {   // J_ab += 2 sum_cd v D_cd
        const int ia = ab / C::NB, ibb = ab - ia * C::NB;
        T v = T(0);
        for (int cd = 0; cd < C::NCD; ++cd) {
          const int ic = cd / C::ND, id = cd - ic * C::ND;
          v = fma_t(I[ab * C::NCD + cd], Dm[(long long)(c0 + ic) * n + d0 + id], v);
        }
        atomicAdd(&Gm[(long long)(a0 + ia) * n + b0 + ibb], widen(T(2) * v));
      }
      for (int cd = lane; a.with_j && cd < C::NCD; cd += 32) {   // J_cd += 2 sum_ab v D_ab
        const int ic = cd / C::ND, id = cd - ic * C::ND;
        T v = T(0);
        for (int ab = 0; ab < C::NAB; ++ab) {
          const int ia = ab / C::NB, ibb = ab - ia * C::NB;
          v = fma_t(I[ab * C::NCD + cd], Dm[(long long)(a0 + ia) * n + b0 + ibb], v);
        }
        atomicAdd(&Gm[(long long)(c0 + ic) * n + d0 + id], widen(T(2) * v));
      }
      for (int e = lane; e < C::NA * C::NC; e += 32) {   // K_ac -= 1/2 sum_bd v D_bd
        const int ia = e / C::NC, ic = e - ia * C::NC;
        T v = T(0);
        for (int ibb = 0; ibb < C::NB; ++ibb)
          for (int id = 0; id < C::ND; ++id)
            v = fma_t(I[(ia * C::NB + ibb) * C::NCD + ic * C::ND + id], Dm[(long long)(b0 + ibb) * n + d0 + id], v);
        atomicAdd(&Gm[(long long)(a0 + ia) * n + c0 + ic], widen(T(-0.5) * v));
      }
      for (int e = lane; e < C::NA * C::ND; e += 32) {   // K_ad -= 1/2 sum_bc v D_bc
        const int ia = e / C::ND, id = e - ia * C::ND;
        T v = T(0);
        for (int ibb = 0; ibb < C::NB; ++ibb)
          for (int ic = 0; ic < C::NC; ++ic)
            v = fma_t(I[(ia * C::NB + ibb) * C::NCD + ic * C::ND + id], Dm[(long long)(b0 + ibb) * n + c0 + ic], v);
        atomicAdd(&Gm[(long long)(a0 + ia) * n + d0 + id], widen(T(-0.5) * v));
      }
      for (int e = lane; e < C::NB * C::NC; e += 32) {   // K_bc -= 1/2 sum_ad v D_ad
        const int ibb = e / C::NC, ic = e - ibb * C::NC;
        T v = T(0);
        for (int ia = 0; ia < C::NA; ++ia)
          for (int id = 0; id < C::ND; ++id)
            v = fma_t(I[(ia * C::NB + ibb) * C::NCD + ic * C::ND + id], Dm[(long long)(a0 + ia) * n + d0 + id], v);
        atomicAdd(&Gm[(long long)(b0 + ibb) * n + c0 + ic], widen(T(-0.5) * v));
      }
      for (int e = lane; e < C::NB * C::ND; e += 32) {   // K_bd -= 1/2 sum_ac v D_ac
        const int ibb = e / C::ND, id = e - ibb * C::ND;
        T v = T(0);
        for (int ia = 0; ia < C::NA; ++ia)
          for (int ic = 0; ic < C::NC; ++ic)
            v = fma_t(I[(ia * C::NB + ibb) * C::NCD + ic * C::ND + id], Dm[(long long)(a0 + ia) * n + c0 + ic], v);
        atomicAdd(&Gm[(long long)(b0 + ibb) * n + d0 + id], widen(T(-0.5) * v));
      }
      __syncwarp();
    }
  }
  if (lane == 0 && a.stats) {
    atomicAdd(&a.stats[0], cnt_q);
    atomicAdd(&a.stats[1], cnt_q * (unsigned long long)C::NOUT);
    atomicAdd(&a.stats[2], cnt_p);
  }
}

template <int LA, int LB, int LC, int LD, typename T>
static gbhf_status launch_jkd_t(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const T* D, double* G,
                                const T* bra, const T* ket, const T* boys, int ntask, int with_j) {
  if (ntask <= 0) return GBHF_OK;
  using C = MDCfg<LA, LB, LC, LD, 0>;
  const size_t smem = TUV_BYTES + (size_t)JKD_WARPS * C::WS * sizeof(T);
  auto kern = k_jkd<LA, LB, LC, LD, T>;
  static bool attr_set = false;
  if (!attr_set) {
    GBHF_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int per_sm = 0;
  GBHF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, JKD_THREADS, smem));
  per_sm = std::max(per_sm, 1);
  const int grid = std::min(c->nsm * per_sm, (ntask + JKD_WARPS - 1) / JKD_WARPS);
  PairData& P = c->pairs;
  JKDArgs<T> a;
  a.tasks = prec == 0 ? c->tasks.tasks64.p : c->tasks.tasks32.p;
  a.range = c->tasks.ranges.p + 4 * combo + 2 * prec;
  a.counter = c->tasks.counters.p + 2 * combo + prec;
  a.pA = P.A.p;
  a.pB = P.B.p;
  a.poff = P.poff.p;
  a.kseg = P.kseg.p;
  a.seg = P.seg_info.p;
  a.bra = bra;
  a.ket = ket;
  a.npp = (long long)P.nprim_pairs;
  a.shell_f0 = c->tasks.f0.p;
  a.pmol = P.mol.p;
  a.mn = c->tasks.mn.p;
  a.moff = c->tasks.moff.p;
  a.sscale = c->tasks.sscale.p;
  a.D = D;
  a.G = G;
  a.boys = boys;
  a.stats = c->tasks.stats.p + 3 * (2 * combo + prec);
  a.with_j = with_j;
  a.Q = P.Q.p;
  a.thr = c->tasks.thr_exact;
  kern<<<grid, JKD_THREADS, smem, strm>>>(a);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

template <typename T>
static gbhf_status launch_jkd_combo(gbhf_ctx* c, cudaStream_t strm, int k, int prec, const T* D, double* G,
                                    const T* bra, const T* ket, const T* boys, int nt, int wj) {
#define GBHF_JKD(K, la, lb, lc, ld) \
  case K: return launch_jkd_t<la, lb, lc, ld, T>(c, strm, k, prec, D, G, bra, ket, boys, nt, wj);
  switch (k) {   // COMBO_BRA / COMBO_KET 6..20; class 3 = ds, 4 = dp, 5 = dd
    GBHF_JKD(6, 2, 0, 0, 0)
    GBHF_JKD(7, 2, 0, 1, 0)
    GBHF_JKD(8, 2, 0, 1, 1)
    GBHF_JKD(9, 2, 0, 2, 0)
    GBHF_JKD(10, 2, 1, 0, 0)
    GBHF_JKD(11, 2, 1, 1, 0)
    GBHF_JKD(12, 2, 1, 1, 1)
    GBHF_JKD(13, 2, 1, 2, 0)
    GBHF_JKD(14, 2, 1, 2, 1)
    GBHF_JKD(15, 2, 2, 0, 0)
    GBHF_JKD(16, 2, 2, 1, 0)
    GBHF_JKD(17, 2, 2, 1, 1)
    GBHF_JKD(18, 2, 2, 2, 0)
    GBHF_JKD(19, 2, 2, 2, 1)
    GBHF_JKD(20, 2, 2, 2, 2)
    default: return fail(c, GBHF_ERR_UNSUPPORTED, "no d-class J/K kernel for combo " + std::to_string(k));
  }
#undef GBHF_JKD
}

gbhf_status launch_jk_dclass(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const double* D64,
                             const float* D32, double* G, int ntask, int with_j) {
  PairData& P = c->pairs;
  if (prec == 0)
    return launch_jkd_combo<double>(c, strm, combo, 0, D64, G, P.bra64.p, P.ket64.p, c->boysh64.p, ntask, with_j);
  return launch_jkd_combo<float>(c, strm, combo, 1, D32, G, P.bra32.p, P.ket32.p, c->boysh32.p, ntask, with_j);
}

// --------------------------------------------------------- Schwarz bounds ----
// Q_AB = sqrt(max_ab |(ab|ab)|) of the scaled components, warp per pair; the
// pairs' primitive data in pair-contiguous field-major layout.
template <int LA, int LB>
__global__ void __launch_bounds__(JKD_THREADS) k_schwarzd(int p0, int p1, const int* __restrict__ pA,
                                                           const int* __restrict__ pB, const int* __restrict__ pK,
                                                           const int* __restrict__ poff,
                                                           const double* __restrict__ bra, long long npp,
                                                           const double* __restrict__ sscale,
                                                           const double* __restrict__ boys, double* __restrict__ Q) {
  using C = MDCfg<LA, LB, LA, LB, 0>;
  extern __shared__ __align__(16) unsigned char jkd_smem[];
  int* tuv = reinterpret_cast<int*>(jkd_smem);
  md_fill_tuv(tuv, C::L);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = p0 + blockIdx.x * JKD_WARPS + warp;
  if (t >= p1) return;
  double* ws = reinterpret_cast<double*>(jkd_smem + TUV_BYTES) + warp * C::WS;
  const int K = pK[t];
  const long long o = poff[t];
  double acc[C::NPL];
#pragma unroll
  for (int k = 0; k < C::NPL; ++k) acc[k] = 0.0;
  for (int kb = 0; kb < K; ++kb) {
    MDPrim<double> bp;
    md_load_prim(bra, npp, o + kb, bp);
    md_bra_e<C>(ws, bp, lane);
    for (int kc = 0; kc < K; ++kc) {
      MDPrim<double> kp;
      md_load_prim(bra, npp, o + kc, kp);
      md_prim_x<C>(ws, tuv, bp, kp, boys, lane);
      md_bra_acc<C>(ws, acc, lane);
      __syncwarp();
    }
  }
  const int A = pA[t], B = pB[t];
  double mx = 0.0;
#pragma unroll
  for (int k = 0; k < C::NPL; ++k) {
    const int e = lane + 32 * k;
    if (e < C::NOUT) {
      const int ab = e / C::NCD, cd = e - ab * C::NCD;
      if (ab == cd) {
        const int ia = ab / C::NB, ibb = ab - ia * C::NB;
        const double sc = sscale[6 * A + ia] * sscale[6 * B + ibb];
        mx = fmax(mx, fabs(acc[k]) * sc * sc);
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if (lane == 0) Q[t] = sqrt(mx);
}

template <int LA, int LB>
static gbhf_status launch_schwarzd(gbhf_ctx* c, int p0, int p1, const int* dA, const int* dB, const int* d_K,
                                   const int* d_poff, const double* d_bra, long long npp, double* d_Q) {
  using C = MDCfg<LA, LB, LA, LB, 0>;
  const size_t smem = TUV_BYTES + (size_t)JKD_WARPS * C::WS * sizeof(double);
  auto kern = k_schwarzd<LA, LB>;
  static bool attr_set = false;
  if (!attr_set) {
    GBHF_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  const int blocks = (p1 - p0 + JKD_WARPS - 1) / JKD_WARPS;
  kern<<<blocks, JKD_THREADS, smem, c->stream>>>(p0, p1, dA, dB, d_K, d_poff, d_bra, npp, c->tasks.sscale.p,
                                                 c->boysh64.p, d_Q);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

gbhf_status schwarz_dclasses_dev(gbhf_ctx* c, const int* cls_start, const int* dA, const int* dB, const int* d_K,
                                 const int* d_poff, const double* d_bra, long long npp, double* d_Q) {
  for (int cl = 3; cl < NPCLS; ++cl) {
    const int p0 = cls_start[cl], p1 = cls_start[cl + 1];
    if (p1 <= p0) continue;
    if (cl == 3) GBHF_TRY((launch_schwarzd<2, 0>(c, p0, p1, dA, dB, d_K, d_poff, d_bra, npp, d_Q)));
    else if (cl == 4) GBHF_TRY((launch_schwarzd<2, 1>(c, p0, p1, dA, dB, d_K, d_poff, d_bra, npp, d_Q)));
    else GBHF_TRY((launch_schwarzd<2, 2>(c, p0, p1, dA, dB, d_K, d_poff, d_bra, npp, d_Q)));
  }
  return GBHF_OK;
}

}  // namespace gbhf
