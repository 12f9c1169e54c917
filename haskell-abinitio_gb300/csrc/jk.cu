// Direct J/K Fock build: screened task lists and per-class ERI+scatter kernels.
//
// Unique shell quartets (AB|CD): bra pair of class X, ket pair of class Y
// with X >= Y, and within one class ket index <= bra index, which visits
// each quartet of the 8-fold permutation orbit once.  With the degeneracy
// weight s = (A==B ? 1/2 : 1)(C==D ? 1/2 : 1)(AB==CD ? 1/2 : 1) every
// component integral v = (ab|cd) adds, to a non-symmetric accumulator G'',
//   G''_ab += 2 s v D_cd,  G''_cd += 2 s v D_ab,
//   G''_ac -= s v D_bd/2,  G''_bc -= s v D_ad/2,  G''_ad -= s v D_bc/2,  G''_bd -= s v D_ac/2,
// and G = G'' + G''^T equals J - K/2 of the reference's calcGmatrix
// (HartreeFock/HartreeFock.hs:225-241): G_ab = sum_kl D_lk [(ab|kl) - (al|kb)/2].
//
// Work decomposition: a task is (bra pair, <= 32 consecutive kets of one ket
// segment); one warp runs one task, lane = ket.  Kets inside a segment share
// the primitive-pair count, so lanes do equal work; the segment is sorted by
// Schwarz bound, so the kets that pass Q_bra Q_ket w >= cutoff form a prefix
// found by binary search, and the FP64/FP32 split of mixed precision is a
// second prefix boundary.  Warps pull tasks from a per-kernel atomic counter
// (no waiting on other warps).
#include <algorithm>
#include <cstring>

#include <type_traits>

#include "gbhf_internal.h"

namespace gbhf {


template <typename T, int N>
struct RegAcc {
  T v[N];
  __device__ __forceinline__ T& operator[](int i) { return v[i]; }
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = T(0);
  }
  __device__ __forceinline__ T get(int i) const { return v[i]; }
};

template <int N>
struct SmemAcc {
  double* p;   // this thread's column, stride blockDim (128)
  __device__ __forceinline__ double& operator[](int i) { return p[i * 128]; }
  __device__ __forceinline__ void zero() {
#pragma unroll 4
    for (int i = 0; i < N; ++i) p[i * 128] = 0.0;
  }
  __device__ __forceinline__ double get(int i) const { return p[i * 128]; }
};

}  // namespace gbhf

#include "eri_gen.cuh"

namespace gbhf {

template <typename T>
struct JKArgs {
  const int4* tasks;
  const int* range;    // [start, end)
  int* counter;
  const int* pA;
  const int* pB;
  const int* pK;
  const int* poff;
  const int* kseg;
  const int4* seg;
  const T* bra;
  const T* ket;
  long long npp;
  const int* shell_f0;         // first function of each shell within its molecule
  const int* pmol;             // molecule of each pair
  const int* mn;               // functions per molecule
  const long long* moff;       // offset of each molecule's block in D and G
  const T* D;                  // stacked n_m x n_m densities
  double* G;                   // stacked n_m x n_m Fock accumulators
  const T* boys;
  unsigned long long* stats;   // [shell quartets, fn quartets, prim quartets]
  const double* sscale;        // per shell 6 component scales (d shells)
  int with_j;                  // 0: exchange only (the open-shell spin-density build)
  const double* Q;             // Schwarz bound of each pair
  const float* Qf;             // the same in FP32
  double thr;                  // drop a quartet when Q_ab Q_cd max|D| over its six density blocks is below
  float thrf;
};

template <int LA, int LB, int LC, int LD>
struct ClassFn;

#define GBHF_CLASS_FN(la, lb, lc, ld, name)                                                              \
  template <>                                                                                            \
  struct ClassFn<la, lb, lc, ld> {                                                                       \
    template <typename T, typename Acc>                                                                  \
    static __device__ __forceinline__ void run(const T* sb, int nbra, int bstep, T q, T invq, T Qx, T Qy, T Qz,  \
                                               T QCx, T QCy, T QCz, T QDx, T QDy, T QDz, T Kcd,           \
                                               const T* boys, Acc& acc) {                                 \
      eri_ketprim_##name<T, Acc>(sb, nbra, bstep, q, invq, Qx, Qy, Qz, QCx, QCy, QCz, QDx, QDy, QDz, Kcd, boys, \
                                 acc);                                                                   \
    }                                                                                                    \
  };
GBHF_CLASS_FN(0, 0, 0, 0, ssss)
GBHF_CLASS_FN(1, 0, 0, 0, psss)
GBHF_CLASS_FN(1, 0, 1, 0, psps)
GBHF_CLASS_FN(0, 0, 1, 1, sspp)
GBHF_CLASS_FN(1, 0, 1, 1, pspp)
GBHF_CLASS_FN(1, 1, 1, 1, pppp)
GBHF_CLASS_FN(2, 0, 0, 0, dsss)
GBHF_CLASS_FN(2, 0, 1, 0, dsps)
GBHF_CLASS_FN(2, 0, 1, 1, dspp)
GBHF_CLASS_FN(2, 0, 2, 0, dsds)
GBHF_CLASS_FN(2, 1, 0, 0, dpss)
GBHF_CLASS_FN(2, 1, 1, 0, dpps)
GBHF_CLASS_FN(2, 2, 0, 0, ddss)

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

constexpr int JK_THREADS = 128;
constexpr int JK_WARPS = JK_THREADS / 32;

template <int LA, int LB, int LC, int LD, typename T, bool SACC>
__global__ void __launch_bounds__(JK_THREADS) k_jk(JKArgs<T> a) {
  constexpr int NA = ncart_c(LA), NB = ncart_c(LB), NC = ncart_c(LC), ND = ncart_c(LD);
  constexpr int NAB = NA * NB, NCD = NC * ND, NOUT = NAB * NCD;
  __shared__ __align__(16) T sbra[JK_WARPS][KMAX_PRIM_PAIRS * BRA_SB];
  __shared__ T sDab[JK_WARPS][NAB > 1 ? NAB : 1];
  extern __shared__ double sacc_dyn[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int start = a.range[0];
  const int ntask = a.range[1] - start;
  unsigned long long cnt_q = 0, cnt_p = 0;
  using AccT = typename std::conditional<SACC, SmemAcc<NOUT>, RegAcc<T, NOUT>>::type;
  AccT acc;
  if constexpr (SACC) acc.p = sacc_dyn + threadIdx.x;
  const long long npp = a.npp;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(a.counter, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntask) break;
    const int4 task = a.tasks[start + t];
    const int ib = task.x;
    // lanes beyond the task's kets split the primitive quartets: kets sit on the
    // low lg bits of the lane (nk <= 2^lg), the rest of the lane is the slice;
    // the nsl slices form an nsb x (nsl / nsb) grid over bra and ket primitives
    const int nk = task.z;
    const int lg = 32 - __clz(max(nk, 1) - 1);   // ceil(log2(nk)), 0 for one ket
    const int nsl = 32 >> lg;
    const int slice = lane >> lg;
    const int jk = task.y + (lane & ((1 << lg) - 1));
    const int kb0 = task.w & 0xffff, Kb = (task.w >> 16) - kb0, pb0 = a.poff[ib] + kb0;
    const int K = a.seg[a.kseg[task.y]].z;   // ket primitive pairs, shared by the task's kets
    // the classes whose per-lane pair has the higher momentum transform it once
    // per call (ket primitive and bra-primitive range): about one primitive
    // quartet of extra work per call
    constexpr int CALLC = (LA + LB < LC + LD) ? 1 : 0;
    // per ket primitive a lane also loads the ket pair's fields and enters the
    // bra loop: about one FP32 primitive quartet of issue slots, next to nothing
    // beside the FP64 arithmetic of an FP64 primitive quartet
    constexpr int KETC = sizeof(T) == 4 ? 1 : 0;
    int lb = 0;
    for (int l = 0, best = 1 << 30; (1 << l) <= nsl; ++l) {   // least work for the busiest lane
      const int cost = (((Kb + (1 << l) - 1) >> l) + CALLC + KETC) * ((K + (nsl >> l) - 1) / (nsl >> l));
      if (KETC ? cost < best : cost <= best) {
        best = cost;
        lb = l;
      }
    }
    const int nsb = 1 << lb, nsk = nsl >> lb;
    const int sb = slice & (nsb - 1), sk = slice >> lb;
    // the molecule's density and Fock blocks (stacked matrices)
    const int mol = a.pmol[ib];
    const int n = a.mn[mol];
    const T* __restrict__ Dm = a.D + a.moff[mol];
    double* __restrict__ Gm = a.G + a.moff[mol];
    const bool active = (lane & ((1 << lg) - 1)) < nk;   // computes
    const bool lead = active && slice == 0;               // scatters
    // bra primitives [kb0, kb1) of pair ib
    const unsigned rkb = (65536u + Kb - 1) / Kb;   // idx / Kb = (idx * rkb) >> 16 for idx < 16 * 36
    for (int idx = lane; idx < BRA_NJK * Kb; idx += 32) {
      const int f = (int)(((unsigned)idx * rkb) >> 16), k = idx - f * Kb;
      sbra[warp][k * BRA_SB + f] = a.bra[(long long)f * npp + pb0 + k];
    }
    const int A = a.pA[ib], B = a.pB[ib];
    const int a0 = a.shell_f0[A], b0 = a.shell_f0[B];
    for (int i = lane; i < NAB; i += 32) sDab[warp][i] = Dm[(long long)(a0 + i / NB) * n + b0 + i % NB];
    __syncwarp();
    acc.zero();
    int C = 0, Dd = 0, c0 = 0, d0 = 0;
    bool keep = false;
    if (active) {
      C = a.pA[jk];
      Dd = a.pB[jk];
      c0 = a.shell_f0[C];
      d0 = a.shell_f0[Dd];
      // exact screening of this quartet: the six density blocks it touches
      // (J: D_ab, D_cd; K: D_ac, D_ad, D_bc, D_bd), tighter than the task lists'
      // per-pair weights (a superposition of atomic densities has zero blocks
      // between atoms, so most quartets of the first build drop here)
      T dmx = T(0);
#pragma unroll
      for (int i = 0; i < NAB; ++i) dmx = fmax_t(dmx, fabs_t(sDab[warp][i]));
#pragma unroll
      for (int ic = 0; ic < NC; ++ic) {
#pragma unroll
        for (int id = 0; id < ND; ++id) dmx = fmax_t(dmx, fabs_t(Dm[(long long)(c0 + ic) * n + d0 + id]));
#pragma unroll
        for (int ia = 0; ia < NA; ++ia) dmx = fmax_t(dmx, fabs_t(Dm[(long long)(a0 + ia) * n + c0 + ic]));
#pragma unroll
        for (int ibb = 0; ibb < NB; ++ibb) dmx = fmax_t(dmx, fabs_t(Dm[(long long)(b0 + ibb) * n + c0 + ic]));
      }
#pragma unroll
      for (int id = 0; id < ND; ++id) {
#pragma unroll
        for (int ia = 0; ia < NA; ++ia) dmx = fmax_t(dmx, fabs_t(Dm[(long long)(a0 + ia) * n + d0 + id]));
#pragma unroll
        for (int ibb = 0; ibb < NB; ++ibb) dmx = fmax_t(dmx, fabs_t(Dm[(long long)(b0 + ibb) * n + d0 + id]));
      }
      if constexpr (sizeof(T) == 4) keep = a.Qf[ib] * a.Qf[jk] * dmx >= a.thrf;   // no FP64-pipe work
      else keep = a.Q[ib] * a.Q[jk] * dmx >= a.thr;
    }
    if (keep) {
      const int4 sg = a.seg[a.kseg[jk]];
      const int len = sg.y - sg.x;
      const long long base = (long long)sg.w + (jk - sg.x);
      const int nbl = sb < Kb ? (Kb - sb + nsb - 1) / nsb : 0;   // this lane's bra primitives
      for (int kc = sk; kc < K; kc += nsk) {
        const long long idx = base + (long long)kc * len;
        const T q = a.ket[BRA_P * npp + idx];
        const T invq = a.ket[BRA_INVP * npp + idx];
        const T Qx = a.ket[BRA_PX * npp + idx], Qy = a.ket[BRA_PY * npp + idx], Qz = a.ket[BRA_PZ * npp + idx];
        T QCx = 0, QCy = 0, QCz = 0, QDx = 0, QDy = 0, QDz = 0;
        if (LC >= 1) {
          QCx = a.ket[BRA_PAX * npp + idx];
          QCy = a.ket[BRA_PAY * npp + idx];
          QCz = a.ket[BRA_PAZ * npp + idx];
        }
        if (LD >= 1) {
          QDx = a.ket[BRA_PBX * npp + idx];
          QDy = a.ket[BRA_PBY * npp + idx];
          QDz = a.ket[BRA_PBZ * npp + idx];
        }
        const T Kcd = a.ket[BRA_K * npp + idx];
        ClassFn<LA, LB, LC, LD>::template run<T, AccT>(sbra[warp] + sb * BRA_SB, nbl, nsb * BRA_SB, q, invq,
                                                       Qx, Qy, Qz, QCx, QCy, QCz, QDx, QDy, QDz, Kcd, a.boys, acc);
      }
      cnt_q += lead && kb0 == 0;
      cnt_p += (unsigned long long)nbl * (sk < K ? (K - sk + nsk - 1) / nsk : 0);
    }
    const bool lead_k = lead && keep;   // scatters
    // warp-uniform: sum the slices (every lane ends with the total of its ket)
    for (int o = 1 << lg; o < 32; o <<= 1) {
#pragma unroll
      for (int i = 0; i < NOUT; ++i) acc[i] += __shfl_xor_sync(0xffffffffu, acc.get(i), o);
    }
    if constexpr (LA == 2 || LB == 2 || LC == 2 || LD == 2) {
      // d shells: the generated code used the first component's coefficients
      if (keep) {
#pragma unroll
        for (int e = 0; e < NOUT; ++e) {
          const int ab = e / NCD, cd = e - ab * NCD;
          T f = T(1);
          if (LA == 2) f *= T(a.sscale[6 * A + ab / NB]);
          if (LB == 2) f *= T(a.sscale[6 * B + ab % NB]);
          if (LC == 2) f *= T(a.sscale[6 * C + cd / ND]);
          if (LD == 2) f *= T(a.sscale[6 * Dd + cd % ND]);
          acc[e] = acc.get(e) * f;
        }
      }
    }
    // ---- scatter into G'' (FP64 atomics)
    const T s = (A == B ? T(0.5) : T(1)) * (C == Dd ? T(0.5) : T(1)) * (ib == jk ? T(0.5) : T(1));
    T dcd[NCD];
#pragma unroll
    for (int ic = 0; ic < NC; ++ic)
#pragma unroll
      for (int id = 0; id < ND; ++id) dcd[ic * ND + id] = lead_k ? Dm[(long long)(c0 + ic) * n + d0 + id] : T(0);
    // J_ab (warp reduce over kets)
    if (a.with_j) {
#pragma unroll
      for (int ab = 0; ab < NAB; ++ab) {
        T v = 0;
#pragma unroll
        for (int cd = 0; cd < NCD; ++cd) v = fma_t(acc.get(ab * NCD + cd), dcd[cd], v);
        v = warp_sum(T(2) * s * v);   // s depends on the lane's ket: apply before the reduction
        if (lane == 0) atomicAdd(&Gm[(long long)(a0 + ab / NB) * n + b0 + ab % NB], widen(v));
      }
    }
    if (lead_k) {
      // J_cd
      if (a.with_j) {
#pragma unroll
        for (int cd = 0; cd < NCD; ++cd) {
          T v = 0;
#pragma unroll
          for (int ab = 0; ab < NAB; ++ab) v = fma_t(acc.get(ab * NCD + cd), sDab[warp][ab], v);
          atomicAdd(&Gm[(long long)(c0 + cd / ND) * n + d0 + cd % ND], widen(T(2) * s * v));
        }
      }
      const T ks = T(-0.5) * s;
      // K_ac -= sum_bd v D_bd ; K_ad -= sum_bc v D_bc
#pragma unroll
      for (int ia = 0; ia < NA; ++ia) {
#pragma unroll
        for (int ic = 0; ic < NC; ++ic) {
          T v = 0;
#pragma unroll
          for (int ibb = 0; ibb < NB; ++ibb)
#pragma unroll
            for (int id = 0; id < ND; ++id)
              v = fma_t(acc.get((ia * NB + ibb) * NCD + ic * ND + id), Dm[(long long)(b0 + ibb) * n + d0 + id], v);
          atomicAdd(&Gm[(long long)(a0 + ia) * n + c0 + ic], widen(ks * v));
        }
#pragma unroll
        for (int id = 0; id < ND; ++id) {
          T v = 0;
#pragma unroll
          for (int ibb = 0; ibb < NB; ++ibb)
#pragma unroll
            for (int ic = 0; ic < NC; ++ic)
              v = fma_t(acc.get((ia * NB + ibb) * NCD + ic * ND + id), Dm[(long long)(b0 + ibb) * n + c0 + ic], v);
          atomicAdd(&Gm[(long long)(a0 + ia) * n + d0 + id], widen(ks * v));
        }
      }
      // K_bc -= sum_ad v D_ad ; K_bd -= sum_ac v D_ac
#pragma unroll
      for (int ibb = 0; ibb < NB; ++ibb) {
#pragma unroll
        for (int ic = 0; ic < NC; ++ic) {
          T v = 0;
#pragma unroll
          for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int id = 0; id < ND; ++id)
              v = fma_t(acc.get((ia * NB + ibb) * NCD + ic * ND + id), Dm[(long long)(a0 + ia) * n + d0 + id], v);
          atomicAdd(&Gm[(long long)(b0 + ibb) * n + c0 + ic], widen(ks * v));
        }
#pragma unroll
        for (int id = 0; id < ND; ++id) {
          T v = 0;
#pragma unroll
          for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ic = 0; ic < NC; ++ic)
              v = fma_t(acc.get((ia * NB + ibb) * NCD + ic * ND + id), Dm[(long long)(a0 + ia) * n + c0 + ic], v);
          atomicAdd(&Gm[(long long)(b0 + ibb) * n + d0 + id], widen(ks * v));
        }
      }
    }
    __syncwarp();
  }
  // statistics (one atomic per warp and counter)
  cnt_q = (unsigned long long)warp_sum((double)cnt_q);
  cnt_p = (unsigned long long)warp_sum((double)cnt_p);
  if (lane == 0 && a.stats) {
    atomicAdd(&a.stats[0], cnt_q);
    atomicAdd(&a.stats[1], cnt_q * (unsigned long long)(NOUT));
    atomicAdd(&a.stats[2], cnt_p);
  }
}

// ------------------------------------------------------- Schwarz bounds ----
// Q_AB = sqrt(max_ab (ab|ab)) for the pairs of one class (bra = ket = pair),
// with the generated FP64 class code; one warp per pair, its primitive pairs
// staged in the warp's slice of shared memory, lanes over (bra primitive,
// slice of the ket primitives) so that pairs with few primitives still fill
// the warp.
constexpr int SCHWARZ_WARPS = 4;   // 4 x 4608 B of staged primitives per block

template <int LA, int LB>
__global__ void __launch_bounds__(SCHWARZ_WARPS * 32) k_schwarz_cls(int p0, int p1, const int* __restrict__ pK,
                                                                     const int* __restrict__ poff,
                                                                     const double* __restrict__ bra, long long npp,
                                                                     const double* __restrict__ boys,
                                                                     double* __restrict__ Q) {
  constexpr int NA = ncart_c(LA), NB = ncart_c(LB), NAB = NA * NB;
  __shared__ __align__(16) double sb[SCHWARZ_WARPS][KMAX_PRIM_PAIRS * BRA_SB];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = p0 + blockIdx.x * SCHWARZ_WARPS + warp;
  if (t >= p1) return;   // whole warps
  const int K = pK[t];
  const long long o = poff[t];
  double* s = sb[warp];
  for (int idx = lane; idx < BRA_NFIELD * K; idx += 32) {
    const int f = idx / K, k = idx - f * K;
    s[k * BRA_SB + f] = bra[f * npp + o + k];
  }
  __syncwarp();
  const int nch = max(1, min(K, 32 / max(K, 1)));
  const int cs = (K + nch - 1) / nch;
  RegAcc<double, NAB * NAB> acc;
  acc.zero();
  for (int it = lane; it < K * nch; it += 32) {
    const int k = it / nch, ch = it - k * nch;
    const int k0 = ch * cs, nk = min(K, k0 + cs) - k0;
    if (nk <= 0) continue;
    auto g = [&](int f) { return s[k * BRA_SB + f]; };
    ClassFn<LA, LB, LA, LB>::template run<double, RegAcc<double, NAB * NAB>>(
        s + k0 * BRA_SB, nk, BRA_SB, g(BRA_P), g(BRA_INVP), g(BRA_PX), g(BRA_PY), g(BRA_PZ), g(BRA_PAX), g(BRA_PAY),
        g(BRA_PAZ), g(BRA_PBX), g(BRA_PBY), g(BRA_PBZ), g(BRA_K), boys, acc);
  }
  double mx = 0;
#pragma unroll
  for (int ab = 0; ab < NAB; ++ab) mx = fmax(mx, fabs(warp_sum(acc.get(ab * NAB + ab))));
  if (lane == 0) Q[t] = sqrt(mx);
}

gbhf_status schwarz_classes_dev(gbhf_ctx* c, const int* cls_start, const int* d_K, const int* d_poff,
                                const double* d_bra, long long npp, double* d_Q) {
  for (int cl = 0; cl < 3; ++cl) {   // s/p classes; jkd.cu has the d classes
    const int p0 = cls_start[cl], p1 = cls_start[cl + 1];
    if (p1 <= p0) continue;
    const int blocks = (p1 - p0 + SCHWARZ_WARPS - 1) / SCHWARZ_WARPS, thr = SCHWARZ_WARPS * 32;
    if (cl == 0)
      k_schwarz_cls<0, 0><<<blocks, thr, 0, c->stream>>>(p0, p1, d_K, d_poff, d_bra, npp, c->boysh64.p, d_Q);
    else if (cl == 1)
      k_schwarz_cls<1, 0><<<blocks, thr, 0, c->stream>>>(p0, p1, d_K, d_poff, d_bra, npp, c->boysh64.p, d_Q);
    else
      k_schwarz_cls<1, 1><<<blocks, thr, 0, c->stream>>>(p0, p1, d_K, d_poff, d_bra, npp, c->boysh64.p, d_Q);
    count_launch(c);
    GBHF_CUDA(c, cudaGetLastError());
  }
  return GBHF_OK;
}

// ------------------------------------------------------------ task lists ----

struct TaskGenArgs {
  int nitems;
  int ncombo;                    // quartet classes (bra pair class, ket pair class)
  int cbra[NCOMBO_MAX], cket[NCOMBO_MAX];
  int all_pairs;                 // every ordered (bra, ket) pair, else each unordered pair once in one class
  int ket_ge[NCOMBO_MAX];        // one class: 1 = (i | j >= i), the bra with more primitives; 0 = (i | j <= i)
  int lane_prims[NCOMBO_MAX];    // per combo: primitive quartets per lane and task (bra split)
  int task_kets[NCOMBO_MAX];     // per combo: kets per task (32: a lane per ket; fewer: a warp per quartet)
  int square_w;                  // bound uses the squared density weight (gradient)
  const int* item_combo_start;   // ncombo+1 item offsets
  const int* cls_start;          // NPCLS+1
  const int* seg_cls_start;      // NPCLS+1
  int nmol;
  const int* pmol;               // molecule of each pair
  const int* mseg;               // ket segments of (class, molecule)
  const int* mact;               // per molecule: 1 = build its quartets (nullptr: all)
  const int4* seg;
  const double* Q;
  const int* pK;                 // primitive pairs per shell pair
  double thr_all, thr64;         // cutoff / weight, mixed cutoff / weight
  const double* pw;              // per-pair density weight (local mode) or nullptr
  const double* sw;              // per-segment max of pw (local mode)
  int* count;                    // 2 per item
  const int* off64;              // exclusive scans (nitems + 1)
  const int* off32;
  int4* tasks64;
  int4* tasks32;
};

__device__ __forceinline__ int count_ge(const double* Q, int lo, int hi, double thr) {
  // Q descending on [lo, hi): number of entries with Q >= thr
  int a = lo, b = hi;
  while (a < b) {
    int m = (a + b) >> 1;
    if (Q[m] >= thr) a = m + 1;
    else b = m;
  }
  return a - lo;
}

template <bool FILL>
__global__ void k_tasks(TaskGenArgs g) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= g.nitems) return;
  int k = 0;
  while (k + 1 < g.ncombo && it >= g.item_combo_start[k + 1]) ++k;
  const int X = g.cbra[k], Y = g.cket[k];
  const int i = g.cls_start[X] + (it - g.item_combo_start[k]);
  const double qi = (g.mact && !g.mact[g.pmol[i]]) ? 0.0 : g.Q[i];   // inactive molecule: no tasks
  int n64 = 0, n32 = 0;
  int w64 = FILL ? g.off64[it] : 0, w32 = FILL ? g.off32[it] : 0;
  const double wi = g.pw ? g.pw[i] : 1.0;
  const int kb = g.pK[i];
  if (qi > 0) {
    const int m = g.pmol[i];
    const int s_lo = g.mseg[2 * (Y * g.nmol + m)], s_hi = g.mseg[2 * (Y * g.nmol + m) + 1];
    for (int sidx = s_lo; sidx < s_hi; ++sidx) {
      const int4 s = g.seg[sidx];
      // bound of (bra|ket) contributions: Q_bra Q_ket max(w_bra, max w over the ket segment)
      double w = g.pw ? fmax(wi, g.sw[sidx]) : 1.0;
      if (g.square_w) w *= w;
      if (!(w > 0)) continue;
      const double ta = g.thr_all / (qi * w), t64 = g.thr64 / (qi * w);
      // one class: each unordered pair of pairs once.  Pairs are sorted by
      // primitive count (descending) within a (class, molecule), so with
      // (i | j >= i) the bra - staged once for the warp - is the pair with
      // more primitives and a lane's ket loop (a load of the ket pair's fields
      // per primitive) is the shorter one; (i | j <= i) the other way round
      int lo = s.x, hi = s.y;
      if (!g.all_pairs && X == Y) {
        if (g.ket_ge[k]) lo = max(lo, i);
        else hi = min(hi, i + 1);
      }
      if (lo >= hi) continue;
      const int keep = count_ge(g.Q, lo, hi, ta);
      int k64 = count_ge(g.Q, lo, lo + keep, t64);
      const int k32 = keep - k64;
      // split the bra primitives so that one lane handles at most about
      // lane_prims primitive quartets per task (bounds the launch tail)
      const int lp = g.lane_prims[k], tk = g.task_kets[k];
      const int nch0 = min(kb, (kb * s.z + lp - 1) / lp);
      const int cs = (kb + nch0 - 1) / nch0;
      const int nch = (kb + cs - 1) / cs;
      if (FILL) {
        for (int ch = 0; ch < nch; ++ch) {
          const int w = (ch * cs) | (min(kb, (ch + 1) * cs) << 16);
          for (int o = 0; o < k64; o += tk) g.tasks64[w64++] = make_int4(i, lo + o, min(tk, k64 - o), w);
          for (int o = 0; o < k32; o += tk) g.tasks32[w32++] = make_int4(i, lo + k64 + o, min(tk, k32 - o), w);
        }
      } else {
        n64 += nch * ((k64 + tk - 1) / tk);
        n32 += nch * ((k32 + tk - 1) / tk);
      }
    }
  }
  if (!FILL) {
    g.count[2 * it] = n64;
    g.count[2 * it + 1] = n32;
  }
}

// Exclusive scans of count[2 i] and count[2 i + 1] into off64 and off32
// (n + 1 entries each) in three launches: tile sums, a one-block scan of the
// tile sums, and the tiles' own scans with their offsets.  A tile is 2048
// items staged in shared memory with coalesced loads; each thread scans 8
// consecutive items.
constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Exclusive block scan of (a, b) over the block's 256 threads; totals in ta, tb.
__device__ __forceinline__ void block_exscan2(int& a, int& b, int& ta, int& tb) {
  __shared__ int wa[SCAN_THREADS / 32], wb[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {
      ia += xa;
      ib += xb;
    }
  }
  if (lane == 31) {
    wa[w] = ia;
    wb[w] = ib;
  }
  __syncthreads();
  int pa = 0, pb = 0;
  ta = 0;
  tb = 0;
  for (int k = 0; k < SCAN_THREADS / 32; ++k) {
    if (k < w) {
      pa += wa[k];
      pb += wb[k];
    }
    ta += wa[k];
    tb += wb[k];
  }
  a = pa + ia - a;
  b = pb + ib - b;
  __syncthreads();
}

__device__ __forceinline__ void scan_load_tile(int n, const int* __restrict__ count, int tile, int* sm) {
  const int base = tile * SCAN_TILE;
  for (int e = threadIdx.x; e < 2 * SCAN_TILE; e += SCAN_THREADS) {
    const int i = base + e / 2;
    sm[e] = i < n ? count[2 * (long)base + e] : 0;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(int n, const int* __restrict__ count,
                                                             int* __restrict__ part) {
  __shared__ int sm[2 * SCAN_TILE];
  scan_load_tile(n, count, blockIdx.x, sm);
  int a = 0, b = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    a += sm[2 * (threadIdx.x * SCAN_ITEMS + k)];
    b += sm[2 * (threadIdx.x * SCAN_ITEMS + k) + 1];
  }
  int ta, tb;
  block_exscan2(a, b, ta, tb);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = ta;
    part[2 * blockIdx.x + 1] = tb;
  }
}

// One block: exclusive scan of the tile sums in place, totals into off64[n], off32[n].
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_parts(int ntile, int n, int* __restrict__ part,
                                                             int* __restrict__ off64, int* __restrict__ off32) {
  int ca = 0, cb = 0;   // carry over chunks of 256 tiles
  for (int t0 = 0; t0 < ntile; t0 += SCAN_THREADS) {
    const int t = t0 + threadIdx.x;
    int a = t < ntile ? part[2 * t] : 0, b = t < ntile ? part[2 * t + 1] : 0;
    int ta, tb;
    block_exscan2(a, b, ta, tb);
    if (t < ntile) {
      part[2 * t] = ca + a;
      part[2 * t + 1] = cb + b;
    }
    ca += ta;
    cb += tb;
  }
  if (threadIdx.x == 0) {
    off64[n] = ca;
    off32[n] = cb;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(int n, const int* __restrict__ count,
                                                             const int* __restrict__ part, int* __restrict__ off64,
                                                             int* __restrict__ off32) {
  __shared__ int sm[2 * SCAN_TILE];
  scan_load_tile(n, count, blockIdx.x, sm);
  int a = 0, b = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    a += sm[2 * (threadIdx.x * SCAN_ITEMS + k)];
    b += sm[2 * (threadIdx.x * SCAN_ITEMS + k) + 1];
  }
  int ta, tb;
  block_exscan2(a, b, ta, tb);
  a += part[2 * blockIdx.x];
  b += part[2 * blockIdx.x + 1];
  const int i0 = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    if (i0 + k < n) {
      off64[i0 + k] = a;
      off32[i0 + k] = b;
    }
    a += sm[2 * (threadIdx.x * SCAN_ITEMS + k)];
    b += sm[2 * (threadIdx.x * SCAN_ITEMS + k) + 1];
  }
}

__global__ void k_ranges(int ncombo, const int* item_combo_start, const int* off64, const int* off32, int* ranges) {
  const int k = threadIdx.x;
  if (k >= ncombo) return;
  ranges[4 * k + 0] = off64[item_combo_start[k]];
  ranges[4 * k + 1] = off64[item_combo_start[k + 1]];
  ranges[4 * k + 2] = off32[item_combo_start[k]];
  ranges[4 * k + 3] = off32[item_combo_start[k + 1]];
}

// Density weights for incremental builds and the gradient: per shell its row
// maximum of |D| over its molecule's functions, per pair w = max(block max of
// the pair, row A, row B) and the block max alone, per ket segment the largest
// block max of its pairs.
__global__ void k_shell_rowmax(int ns, const int* __restrict__ f0, const int* __restrict__ nc,
                               const int* __restrict__ smol, const int* __restrict__ mn,
                               const long long* __restrict__ moff, const double* __restrict__ D,
                               double* __restrict__ row) {
  const int s = blockIdx.x;
  if (s >= ns) return;
  const int m = smol[s], n = mn[m];
  const double* Dm = D + moff[m];
  double v = 0;
  for (int a = 0; a < nc[s]; ++a)
    for (int j = threadIdx.x; j < n; j += blockDim.x) v = fmax(v, fabs(Dm[(long)(f0[s] + a) * n + j]));
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = fmax(v, sh[w]);
    row[s] = v;
  }
}

// A quartet (AB|CD) feeds J_AB (dD_CD), J_CD (dD_AB) and K_AC, K_AD, K_BC, K_BD
// (dD_BD, dD_BC, dD_AD, dD_AC); every exchange block holds a bra shell, so
// max(pw[bra], pb[ket]) bounds all six density factors.
__global__ void k_pair_weight(int np, const int* __restrict__ pA, const int* __restrict__ pB,
                              const int* __restrict__ pmol, const int* __restrict__ f0, const int* __restrict__ nc,
                              const int* __restrict__ mn, const long long* __restrict__ moff,
                              const double* __restrict__ D, const double* __restrict__ row, double* __restrict__ pw,
                              double* __restrict__ pb) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int A = pA[p], B = pB[p], m = pmol[p], n = mn[m];
  const double* Dm = D + moff[m];
  double b = 0;
  for (int x = 0; x < nc[A]; ++x)
    for (int y = 0; y < nc[B]; ++y) b = fmax(b, fabs(Dm[(long)(f0[A] + x) * n + f0[B] + y]));
  pw[p] = fmax(b, fmax(row[A], row[B]));
  pb[p] = b;
}

__global__ void k_seg_max(int nseg, const int4* __restrict__ seg, const double* __restrict__ pw, double* __restrict__ sw) {
  const int s = blockIdx.x;
  if (s >= nseg) return;
  const int4 g = seg[s];
  double m = 0;
  for (int p = g.x + threadIdx.x; p < g.y; p += blockDim.x) m = fmax(m, pw[p]);
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, sh[w]);
    sw[s] = m;
  }
}

static gbhf_status density_weights(gbhf_ctx* c, TaskLists& st, const double* d_dD) {
  PairData& P = c->pairs;
  const TaskLists& sh = c->tasks;   // per-shell and per-molecule arrays
  const int ns = (int)c->basis.shells.size();
  GBHF_CUDA(c, st.row.alloc(ns));
  GBHF_CUDA(c, st.pw.alloc(std::max(P.npairs, 1)));
  GBHF_CUDA(c, st.pb.alloc(std::max(P.npairs, 1)));
  GBHF_CUDA(c, st.sw.alloc(std::max(P.nseg_total, 1)));
  k_shell_rowmax<<<ns, 128, 0, c->stream>>>(ns, sh.f0.p, sh.nc.p, sh.smol.p, sh.mn.p, sh.moff.p, d_dD, st.row.p);
  k_pair_weight<<<(P.npairs + 127) / 128, 128, 0, c->stream>>>(P.npairs, P.A.p, P.B.p, P.mol.p, sh.f0.p, sh.nc.p,
                                                               sh.mn.p, sh.moff.p, d_dD, st.row.p, st.pw.p, st.pb.p);
  if (P.nseg_total > 0) k_seg_max<<<P.nseg_total, 256, 0, c->stream>>>(P.nseg_total, P.seg_info.p, st.pb.p, st.sw.p);
  count_launch(c, 3);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// Quartet-class task lists of TL for the combos (cbra[k], cket[k]).
static gbhf_status build_task_lists(gbhf_ctx* c, TaskLists& TL, int ncombo, const int* cbra, const int* cket,
                                    const int* lane_prims, const int* task_kets, bool all_pairs, bool square_w,
                                    double thr_all, double thr64, const double* pw, const double* sw) {
  PairData& P = c->pairs;
  int* h_ranges = TL.hranges;
  std::vector<int> ics(ncombo + 1, 0);
  for (int k = 0; k < ncombo; ++k) {
    const int X = cbra[k];
    ics[k + 1] = ics[k] + (P.cls_start[X + 1] - P.cls_start[X]);
  }
  TL.nitems = ics[ncombo];
  TL.combo_item_start = ics;
  TL.ncombo = ncombo;
  const int ni = TL.nitems;
  DBuf<int>& d_ics = TL.ics_d;
  DBuf<int>& d_cls = TL.cls_d;
  DBuf<int>& d_scs = TL.scs_d;
  GBHF_CUDA(c, d_ics.alloc(ncombo + 1));
  GBHF_CUDA(c, d_cls.alloc(NPCLS + 1));
  GBHF_CUDA(c, d_scs.alloc(NPCLS + 1));
  GBHF_CUDA(c, cudaMemcpyAsync(d_ics.p, ics.data(), (ncombo + 1) * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(d_cls.p, P.cls_start, (NPCLS + 1) * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(d_scs.p, P.seg_cls_start, (NPCLS + 1) * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, TL.item_count.alloc(2 * (size_t)std::max(ni, 1)));
  GBHF_CUDA(c, TL.item_off.alloc(2 * ((size_t)ni + 1)));
  GBHF_CUDA(c, TL.ranges.alloc(4 * ncombo));
  GBHF_CUDA(c, TL.counters.alloc(2 * ncombo));
  GBHF_CUDA(c, TL.stats.alloc(3 * 2 * ncombo));
  int* off64 = TL.item_off.p;
  int* off32 = TL.item_off.p + ni + 1;
  TaskGenArgs g;
  g.nitems = ni;
  g.ncombo = ncombo;
  for (int k = 0; k < NCOMBO_MAX; ++k) {
    g.cbra[k] = k < ncombo ? cbra[k] : 0;
    g.cket[k] = k < ncombo ? cket[k] : 0;
    g.lane_prims[k] = k < ncombo ? std::max(1, lane_prims[k]) : 1;
    g.task_kets[k] = k < ncombo ? std::min(32, std::max(1, task_kets[k])) : 32;
    // the (ss|ss) and (ps|ps) quartets with the bra of more primitives: the
    // FP32 launches gain 13-14% (fewer ket-field loads per primitive
    // quartet); (pp|pp) FP64 lost 18% that way (its launch is tail-bound)
    g.ket_ge[k] = k < ncombo && cbra[k] == cket[k] && cbra[k] <= 1 ? 1 : 0;
  }
  g.all_pairs = all_pairs ? 1 : 0;
  g.square_w = square_w ? 1 : 0;
  g.item_combo_start = d_ics.p;
  g.cls_start = d_cls.p;
  g.seg_cls_start = d_scs.p;
  g.seg = P.seg_info.p;
  g.Q = P.Q.p;
  g.pK = P.K.p;
  g.nmol = c->basis.nmol;
  g.pmol = P.mol.p;
  g.mseg = P.mseg.p;
  g.mact = c->mol_active;
  g.thr_all = thr_all;
  g.thr64 = thr64;
  g.pw = pw;
  g.sw = sw;
  g.count = TL.item_count.p;
  g.off64 = off64;
  g.off32 = off32;
  g.tasks64 = nullptr;
  g.tasks32 = nullptr;
  if (ni > 0) {
    k_tasks<false><<<(ni + 127) / 128, 128, 0, c->stream>>>(g);
    count_launch(c);
  }
  {
    const int ntile = std::max(1, (ni + SCAN_TILE - 1) / SCAN_TILE);
    GBHF_CUDA(c, TL.scan_part.alloc(2 * (size_t)ntile));
    k_scan_tiles<<<ntile, SCAN_THREADS, 0, c->stream>>>(ni, TL.item_count.p, TL.scan_part.p);
    k_scan_parts<<<1, SCAN_THREADS, 0, c->stream>>>(ntile, ni, TL.scan_part.p, off64, off32);
    k_scan_apply<<<ntile, SCAN_THREADS, 0, c->stream>>>(ni, TL.item_count.p, TL.scan_part.p, off64, off32);
    count_launch(c, 3);
  }
  // the per-class ranges follow from the offsets alone: one copy and one
  // synchronisation give the host both the ranges and the list sizes
  k_ranges<<<1, 64, 0, c->stream>>>(ncombo, d_ics.p, off64, off32, TL.ranges.p);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  GBHF_CUDA(c, cudaMemcpyAsync(h_ranges, TL.ranges.p, 4 * ncombo * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  const int tot[2] = {ncombo > 0 ? h_ranges[4 * (ncombo - 1) + 1] : 0, ncombo > 0 ? h_ranges[4 * (ncombo - 1) + 3] : 0};
  GBHF_CUDA(c, TL.tasks64.alloc(std::max(tot[0], 1)));
  GBHF_CUDA(c, TL.tasks32.alloc(std::max(tot[1], 1)));
  g.tasks64 = TL.tasks64.p;
  g.tasks32 = TL.tasks32.p;
  if (ni > 0) {
    k_tasks<true><<<(ni + 127) / 128, 128, 0, c->stream>>>(g);
    count_launch(c);
  }
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// d combos evaluated by the generated lane-per-ket code (few components per
// quartet); the others go to the warp-per-quartet kernels of jkd.cu.
static bool gen_dclass(int k) { return (k >= 6 && k <= 11) || k == 15; }

// Default task budgets.  J/K (which 0): lane_prims bounds the primitive
// quartets one lane evaluates in one task, per class (ss|ss) (ps|ss) (ps|ps)
// (pp|ss) (pp|ps) (pp|pp) ...: about the same arithmetic per task, so that the
// longest task - the tail of a persistent launch - stays short ((ss|ss) and
// (ps|ss) take less than that: their launches are short, so the tail is a
// larger share of them, while more tasks cost the overlapped SCF next to
// nothing - 0.1 ms of 48 on (H2O)16/6-31G).  A task never
// splits the ket primitives, so a lane always evaluates at least K_ket of them.
// For the warp-per-quartet d classes it bounds the primitive quartets of one
// quartet in one task, and such a task holds one quartet (a launch then spreads
// its quartets over every resident warp).  Gradient (which 1): the derivative
// code does about twice the ERI work per primitive quartet.
void default_budgets(gbhf_ctx* c, int which) {
  static const int jk_lp[NCOMBO] = {96, 64, 48, 96, 32, 8, 48, 16, 8, 8, 16, 8, 36, 36, 36, 16, 36, 36,
                                    36, 36, 36};
  static const int jk_tk[NCOMBO] = {32, 32, 32, 32, 32, 32, 32, 32, 32, 32, 32, 32, 1, 1, 1, 32, 1, 1, 1, 1, 1};
  static const int gr_lp_sp[NGCOMBO_SP] = {128, 64, 24, 64, 24, 8, 24, 8, 4};
  for (int k = 0; k < NCOMBO_MAX; ++k) {
    if (which == 0) {
      c->jk_lp[k] = k < NCOMBO ? jk_lp[k] : 1;
      c->jk_tk[k] = k < NCOMBO ? jk_tk[k] : 32;
    } else {
      c->gr_lp[k] = k < NGCOMBO_SP ? gr_lp_sp[k] : (grad_gen_combo(k) ? 8 : 36);
      c->gr_tk[k] = grad_gen_combo(k) ? 32 : 1;
    }
  }
}

// Kets per task: 32 (a lane per ket) for the lane-per-ket classes, else free.
bool lane_per_ket(int which, int k) {
  return which == 0 ? (k < NCOMBO_SP || gen_dclass(k)) : grad_gen_combo(k);
}

// J/K lists: the classes with bra class >= ket class, unique quartets, with
// the context's task budgets.
static gbhf_status build_tasks(gbhf_ctx* c, double thr_all, double thr64, const double* pw = nullptr,
                               const double* sw = nullptr) {
  return build_task_lists(c, c->tasks, NCOMBO, COMBO_BRA, COMBO_KET, c->jk_lp, c->jk_tk, false, false, thr_all,
                          thr64, pw, sw);
}

gbhf_status ensure_shell_arrays(gbhf_ctx* c) {
  TaskLists& st = c->tasks;
  if (st.f0_gen == c->basis_gen) return GBHF_OK;
  const Basis& b = c->basis;
  const size_t ns = b.shells.size();
  std::vector<int> f0(ns), nc(ns), at(ns), sm(ns);
  std::vector<double> sc(6 * std::max<size_t>(ns, 1), 1.0);
  for (size_t s = 0; s < ns; ++s) {
    f0[s] = b.shells[s].f0 - b.mol_fn_off[b.shells[s].mol];   // first function within its molecule
    nc[s] = b.shells[s].ncomp;
    at[s] = b.shells[s].atom;
    sm[s] = b.shells[s].mol;
    for (int k = 0; k < 6; ++k) sc[6 * s + k] = b.shells[s].scale[k];
  }
  std::vector<int> mn(b.nmol), fmol(b.nbf), amol(b.natoms);
  for (int m = 0; m < b.nmol; ++m) {
    mn[m] = b.mol_fn_off[m + 1] - b.mol_fn_off[m];
    for (int i = b.mol_fn_off[m]; i < b.mol_fn_off[m + 1]; ++i) fmol[i] = m;
    for (int a = b.mol_atom_off[m]; a < b.mol_atom_off[m + 1]; ++a) amol[a] = m;
  }
  GBHF_CUDA(c, st.f0.alloc(ns));
  GBHF_CUDA(c, st.sscale.alloc(sc.size()));
  GBHF_CUDA(c, st.nc.alloc(ns));
  GBHF_CUDA(c, st.atom.alloc(ns));
  GBHF_CUDA(c, st.smol.alloc(ns));
  GBHF_CUDA(c, st.mn.alloc(b.nmol));
  GBHF_CUDA(c, st.moff.alloc(b.nmol + 1));
  GBHF_CUDA(c, st.fmol.alloc(b.nbf));
  GBHF_CUDA(c, st.amol.alloc(b.natoms));
  GBHF_CUDA(c, st.mfo.alloc(b.nmol + 1));
  GBHF_CUDA(c, st.mao.alloc(b.nmol + 1));
  GBHF_CUDA(c, cudaMemcpyAsync(st.f0.p, f0.data(), ns * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.sscale.p, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.nc.p, nc.data(), ns * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.atom.p, at.data(), ns * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.smol.p, sm.data(), ns * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.mn.p, mn.data(), b.nmol * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.moff.p, b.mol_moff.data(), (b.nmol + 1) * sizeof(long long),
                               cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.fmol.p, fmol.data(), b.nbf * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.amol.p, amol.data(), b.natoms * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.mfo.p, b.mol_fn_off.data(), (b.nmol + 1) * sizeof(int), cudaMemcpyHostToDevice,
                               c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(st.mao.p, b.mol_atom_off.data(), (b.nmol + 1) * sizeof(int), cudaMemcpyHostToDevice,
                               c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  st.f0_gen = c->basis_gen;
  return GBHF_OK;
}

// Gradient lists: every (bra class, ket class) combination, every ordered pair
// of shell pairs, bound Q_bra Q_ket max(w_bra, w_ket)^2 with the pair weights
// of D (|Gamma_abcd| <= that squared weight).
gbhf_status build_grad_tasks(gbhf_ctx* c, const double* d_D, double cutoff, double mixed_cutoff, int precision) {
  GBHF_TRY(ensure_pairs(c));
  GBHF_TRY(ensure_shell_arrays(c));
  TaskLists& gt = c->gtasks;
  GBHF_TRY(density_weights(c, gt, d_D));
  const double t64 = precision == GBHF_PREC_FP64 ? 0.0 : mixed_cutoff;
  GBHF_TRY(build_task_lists(c, gt, NCOMBO_MAX, GRAD_COMBO_BRA, GRAD_COMBO_KET, c->gr_lp, c->gr_tk, true, true,
                            cutoff, t64, gt.pw.p, gt.sw.p));
  return GBHF_OK;
}

template <int LA, int LB, int LC, int LD, typename T, bool SACC>
static gbhf_status launch_class(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const T* D, double* G,
                                const T* bra, const T* ket, const T* boys, const int* f0, int ntask, int with_j) {
  if (ntask <= 0) return GBHF_OK;
  constexpr int NOUT = ncart_c(LA) * ncart_c(LB) * ncart_c(LC) * ncart_c(LD);
  const size_t smem = SACC ? (size_t)NOUT * JK_THREADS * sizeof(double) : 0;
  auto kern = k_jk<LA, LB, LC, LD, T, SACC>;
  static bool attr_set = false;
  if (SACC && !attr_set) {
    GBHF_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int per_sm = 0;
  GBHF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, JK_THREADS, smem));
  per_sm = std::max(per_sm, 1);
  int grid = std::min(c->nsm * per_sm, (ntask + JK_WARPS - 1) / JK_WARPS);
  PairData& P = c->pairs;
  JKArgs<T> a;
  a.tasks = prec == 0 ? c->tasks.tasks64.p : c->tasks.tasks32.p;
  a.range = c->tasks.ranges.p + 4 * combo + 2 * prec;
  a.counter = c->tasks.counters.p + 2 * combo + prec;
  a.pA = P.A.p;
  a.pB = P.B.p;
  a.pK = P.K.p;
  a.poff = P.poff.p;
  a.kseg = P.kseg.p;
  a.seg = P.seg_info.p;
  a.bra = bra;
  a.ket = ket;
  a.npp = (long long)P.nprim_pairs;
  a.shell_f0 = f0;
  a.pmol = P.mol.p;
  a.mn = c->tasks.mn.p;
  a.moff = c->tasks.moff.p;
  a.D = D;
  a.G = G;
  a.boys = boys;
  a.stats = c->tasks.stats.p + 3 * (2 * combo + prec);
  a.sscale = c->tasks.sscale.p;
  a.with_j = with_j;
  a.Q = P.Q.p;
  a.Qf = P.Qf.p;
  a.thr = c->tasks.thr_exact;
  a.thrf = (float)c->tasks.thr_exact;
  kern<<<grid, JK_THREADS, smem, strm>>>(a);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}


gbhf_status jk_build(gbhf_ctx* c, const double* d_Dsq, double* d_G, int precision, double schwarz,
                     double mixed_cutoff, double weight, bool local_weights, bool with_j) {
  const int wj = with_j ? 1 : 0;
  c->tasks.thr_exact = schwarz;   // per-quartet test in the kernels, on the density passed here
  GBHF_TRY(ensure_pairs(c));
  const int n = c->basis.nbf;
  TaskLists& st = c->tasks;
  GBHF_TRY(ensure_shell_arrays(c));
  if (local_weights) {
    // incremental build: bounds weighted by the local size of the density change
    GBHF_TRY(density_weights(c, st, d_Dsq));
    const double t64 = precision == GBHF_PREC_FP64 ? 0.0 : mixed_cutoff;
    GBHF_TRY(build_tasks(c, schwarz, t64, st.pw.p, st.sw.p));
    st.thr_all = -1;   // lists no longer match a uniform weight
    st.thr64 = -1;
  } else {
    if (!(weight > 0)) weight = 1e-300;
    const double thr_all = schwarz / weight;
    const double thr64 = precision == GBHF_PREC_FP64 ? 0.0 : mixed_cutoff / weight;
    if (thr_all != st.thr_all || thr64 != st.thr64 || !c->tasks.tasks64.p) {
      GBHF_TRY(build_tasks(c, thr_all, thr64));
      st.thr_all = thr_all;
      st.thr64 = thr64;
    }
  }
  GBHF_CUDA(c, cudaMemsetAsync(c->tasks.counters.p, 0, 2 * NCOMBO * sizeof(int), c->stream));
  if (!st.stats_pending) {   // the counters add up over builds until flush_jk_stats reads them
    GBHF_CUDA(c, cudaMemsetAsync(c->tasks.stats.p, 0, 6 * NCOMBO * sizeof(unsigned long long), c->stream));
    st.stats_pending = true;
  }
  bool any32 = false;
  for (int k = 0; k < NCOMBO; ++k) any32 |= st.hranges[4 * k + 3] > st.hranges[4 * k + 2];
  if (any32) {
    const size_t nst = (size_t)c->basis.stacked;   // all molecules' blocks
    GBHF_CUDA(c, c->dfloat.alloc(nst));
    GBHF_TRY(to_float(c, nst, d_Dsq, c->dfloat.p));
  }
  PairData& P = c->pairs;
  const int* f0 = st.f0.p;
  int nt[NCOMBO][2];
  for (int k = 0; k < NCOMBO; ++k) {
    nt[k][0] = st.hranges[4 * k + 1] - st.hranges[4 * k + 0];
    nt[k][1] = st.hranges[4 * k + 3] - st.hranges[4 * k + 2];
  }
  const bool ev = c->prof.events;
  // heaviest class first; FP64 lists, then FP32 lists.  Without per-class
  // profiling events the launches go round-robin to the side streams: each is a
  // persistent grid that fills the GPU, and the next one takes over SMs as the
  // tail of the previous one drains.  With profiling events they run in order
  // on the context stream so that each launch is timed alone.
  static const int order[NCOMBO] = {20, 19, 18, 17, 16, 15, 14, 13, 12, 11, 10, 9, 8, 7, 6, 5, 4, 3, 2, 1, 0};
  int ne = 0, nl = 0;
  int ev_combo[2 * NCOMBO], ev_prec[2 * NCOMBO];
  if (ev) GBHF_CUDA(c, cudaEventRecord(c->evc[ne], c->stream));
  else {
    GBHF_CUDA(c, cudaEventRecord(c->fork_ev, c->stream));
    for (int i = 0; i < gbhf_ctx::NSIDE; ++i) GBHF_CUDA(c, cudaStreamWaitEvent(c->side[i], c->fork_ev, 0));
  }
  for (int prec = 0; prec < 2; ++prec) {
    if (prec == 1 && !any32) break;
    const double* D64 = d_Dsq;
    const float* D32 = c->dfloat.p;
    for (int oi = 0; oi < NCOMBO; ++oi) {
      const int k = order[oi];
      if (nt[k][prec] <= 0) continue;
      gbhf_status s = GBHF_OK;
      cudaStream_t strm = ev ? c->stream : c->side[nl % gbhf_ctx::NSIDE];
      ++nl;
      if (k >= NCOMBO_SP && !gen_dclass(k)) {
        s = launch_jk_dclass(c, strm, k, prec, D64, D32, d_G, nt[k][prec], wj);
      } else if (prec == 0) {
        switch (k) {
          case 6: s = launch_class<2, 0, 0, 0, double, false>(c, strm, 6, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[6][0], wj); break;
          case 7: s = launch_class<2, 0, 1, 0, double, false>(c, strm, 7, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[7][0], wj); break;
          case 8: s = launch_class<2, 0, 1, 1, double, true>(c, strm, 8, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[8][0], wj); break;
          case 9: s = launch_class<2, 0, 2, 0, double, true>(c, strm, 9, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[9][0], wj); break;
          case 10: s = launch_class<2, 1, 0, 0, double, false>(c, strm, 10, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[10][0], wj); break;
          case 11: s = launch_class<2, 1, 1, 0, double, true>(c, strm, 11, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[11][0], wj); break;
          case 15: s = launch_class<2, 2, 0, 0, double, true>(c, strm, 15, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[15][0], wj); break;
          case 5: s = launch_class<1, 1, 1, 1, double, true>(c, strm, 5, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[5][0], wj); break;
          case 4: s = launch_class<1, 0, 1, 1, double, false>(c, strm, 4, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[4][0], wj); break;
          case 3: s = launch_class<0, 0, 1, 1, double, false>(c, strm, 3, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[3][0], wj); break;
          case 2: s = launch_class<1, 0, 1, 0, double, false>(c, strm, 2, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[2][0], wj); break;
          case 1: s = launch_class<1, 0, 0, 0, double, false>(c, strm, 1, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[1][0], wj); break;
          default: s = launch_class<0, 0, 0, 0, double, false>(c, strm, 0, 0, D64, d_G, P.bra64.p, P.ket64.p, c->boysh64.p, f0, nt[0][0], wj); break;
        }
      } else {
        switch (k) {
          case 6: s = launch_class<2, 0, 0, 0, float, false>(c, strm, 6, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[6][1], wj); break;
          case 7: s = launch_class<2, 0, 1, 0, float, false>(c, strm, 7, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[7][1], wj); break;
          case 8: s = launch_class<2, 0, 1, 1, float, false>(c, strm, 8, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[8][1], wj); break;
          case 9: s = launch_class<2, 0, 2, 0, float, false>(c, strm, 9, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[9][1], wj); break;
          case 10: s = launch_class<2, 1, 0, 0, float, false>(c, strm, 10, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[10][1], wj); break;
          case 11: s = launch_class<2, 1, 1, 0, float, false>(c, strm, 11, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[11][1], wj); break;
          case 15: s = launch_class<2, 2, 0, 0, float, false>(c, strm, 15, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[15][1], wj); break;
          case 5: s = launch_class<1, 1, 1, 1, float, false>(c, strm, 5, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[5][1], wj); break;
          case 4: s = launch_class<1, 0, 1, 1, float, false>(c, strm, 4, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[4][1], wj); break;
          case 3: s = launch_class<0, 0, 1, 1, float, false>(c, strm, 3, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[3][1], wj); break;
          case 2: s = launch_class<1, 0, 1, 0, float, false>(c, strm, 2, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[2][1], wj); break;
          case 1: s = launch_class<1, 0, 0, 0, float, false>(c, strm, 1, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[1][1], wj); break;
          default: s = launch_class<0, 0, 0, 0, float, false>(c, strm, 0, 1, D32, d_G, P.bra32.p, P.ket32.p, c->boysh32.p, f0, nt[0][1], wj); break;
        }
      }
      if (s != GBHF_OK) return s;
      if (ev) {
        ev_combo[ne] = k;
        ev_prec[ne] = prec;
        ++ne;
        GBHF_CUDA(c, cudaEventRecord(c->evc[ne], c->stream));
      }
    }
  }
  if (!ev) {
    for (int i = 0; i < gbhf_ctx::NSIDE; ++i) {
      GBHF_CUDA(c, cudaEventRecord(c->join_ev[i], c->side[i]));
      GBHF_CUDA(c, cudaStreamWaitEvent(c->stream, c->join_ev[i], 0));
    }
  }
  // statistics: read with the per-class event times when those are taken,
  // else when the profile is read (no host synchronisation per build)
  if (!ev) return GBHF_OK;
  GBHF_TRY(flush_jk_stats(c));
  for (int e = 0; e < ne; ++e) {
    float ms = 0;
    GBHF_CUDA(c, cudaEventElapsedTime(&ms, c->evc[e], c->evc[e + 1]));
    c->prof.cls[ev_combo[e]][ev_prec[e]][3] += ms;
    (ev_prec[e] == 0 ? c->prof.jk_ms64 : c->prof.jk_ms32) += ms;
  }
  return GBHF_OK;
}

gbhf_status flush_jk_stats(gbhf_ctx* c) {
  TaskLists& st = c->tasks;
  if (!st.stats_pending) return GBHF_OK;
  unsigned long long hs[6 * NCOMBO];
  GBHF_CUDA(c, cudaMemcpyAsync(hs, st.stats.p, sizeof(hs), cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  st.stats_pending = false;
  for (int k = 0; k < NCOMBO; ++k)
    for (int p = 0; p < 2; ++p) {
      const unsigned long long* s = hs + 3 * (2 * k + p);
      c->prof.shellq += (double)s[0];
      c->prof.fnq += (double)s[1];
      (p == 0 ? c->prof.prim64 : c->prof.prim32) += (double)s[2];
      c->prof.cls[k][p][0] += (double)s[0];
      c->prof.cls[k][p][1] += (double)s[1];
      c->prof.cls[k][p][2] += (double)s[2];
    }
  return GBHF_OK;
}

}  // namespace gbhf
