// Analytic RHF nuclear gradient (the backward call).
//
// dE/dR_K = sum_ab D_ab dH_ab/dR_K + 1/2 sum_abcd Gamma_abcd d(ab|cd)/dR_K
//           - sum_ab W_ab dS_ab/dR_K + dV_nn/dR_K
// with D = 2 C_occ C_occ^T, W = 2 sum_i eps_i C_i C_i^T and
// Gamma_abcd = D_ab D_cd - (D_ac D_bd + D_ad D_bc)/4.  This is the gradient
// the reference's (uncompiled) energyGradient (HartreeFock/Derivatives.hs:40-48)
// intends, including the Hellmann-Feynman operator term that it zeroes
// (Derivatives.hs:144).  Derivatives of primitive Gaussians follow
// d/dA_x [x_A^i exp(-a r_A^2)] = 2a x_A^(i+1) exp(..) - i x_A^(i-1) exp(..)
// (as calcDervCGF, Derivatives.hs:246-257), applied to the Hermite expansion
// coefficients: dE^(ij)_t/dA_x = 2a E^(i+1,j)_t - i E^(i-1,j)_t.
// Translational invariance gives the fourth centre of an ERI and the
// operator centre of a nuclear-attraction integral.
//
// Open shell (UHF): with D = D_a + D_b, D_s = D_a - D_b and
// W = sum_s C_s,occ eps_s C_s,occ^T, the two-electron density is
// Gamma = D_ab D_cd - (D_a,ac D_a,bd + D_b,ac D_b,bd + D_a,ad D_a,bc + D_b,ad D_b,bc)/2
//       = Gamma_RHF(D) - (D_s,ac D_s,bd + D_s,ad D_s,bc)/4,
// so the kernels run twice: on D as above, and on D_s with the Coulomb
// weight jcoef = 0 (gradient_uhf_dev).
#include <algorithm>
#include <cmath>
#include <vector>

#include "gbhf_internal.h"
#include "gbhf_md.cuh"
#include "grad_gen.cuh"

namespace gbhf {

// ----------------------------------------------------------- two-electron ----
// Warp per task (bra shell pair, up to 32 kets of one segment, a range of bra
// primitives), as the J/K kernels: the bra primitive pairs are staged in
// shared memory, each lane runs the generated bra-derivative code for its ket
// pair against them, and the warp reduces the six bra-centre components before
// one set of atomics.  Summed over every ordered pair of shell pairs with
// weights (2 - delta_AB)(2 - delta_CD), the bra-centre derivatives give the
// whole two-electron gradient (the ket-centre terms of (P|Q) are the
// bra-centre terms of (Q|P)).

constexpr int GR_THREADS = 128;
constexpr int GR_WARPS = GR_THREADS / 32;

template <typename T, int N>
struct GamReg {
  T v[N];
  __device__ __forceinline__ T get(int i) const { return v[i]; }
  __device__ __forceinline__ void set(int i, T x) { v[i] = x; }
};
template <typename T, int N>
struct GamSmem {   // per-thread column of a [N][GR_THREADS] shared array
  T* p;
  // volatile: a read stays where the code places it (the bra loop reads T_ab
  // block by block; hoisted out of the loop, all of T would be live at once)
  __device__ __forceinline__ T get(int i) const { return *(volatile const T*)(p + i * GR_THREADS); }
  __device__ __forceinline__ void set(int i, T x) { p[i * GR_THREADS] = x; }
};

template <int LA, int LB, int LC, int LD>
struct GradFn;
#define GBHF_GRAD_FN(la, lb, lc, ld, name)                                                                      \
  template <>                                                                                                  \
  struct GradFn<la, lb, lc, ld> {                                                                              \
    template <typename T, typename G, typename TK>                                                             \
    static __device__ __forceinline__ void ket(T invq, T QCx, T QCy, T QCz, T QDx, T QDy, T QDz, const G& gam, \
                                               TK& tk) {                                                       \
      grad_ket_##name<T, G, TK>(invq, QCx, QCy, QCz, QDx, QDy, QDz, gam, tk);                                  \
    }                                                                                                          \
    template <typename T, typename TK>                                                                         \
    static __device__ __forceinline__ void run(const T* sb, int nbra, int bstep, T q, T Qx, T Qy, T Qz, T Kcd, \
                                               const T* boys, const TK& tk, T* g) {                            \
      grad_ketprim_##name<T, TK>(sb, nbra, bstep, q, Qx, Qy, Qz, Kcd, boys, tk, g);                            \
    }                                                                                                          \
  };
GBHF_GRAD_FN(0, 0, 2, 0, ssds)
GBHF_GRAD_FN(0, 0, 2, 1, ssdp)
GBHF_GRAD_FN(1, 0, 2, 0, psds)
GBHF_GRAD_FN(2, 0, 0, 0, dsss)
GBHF_GRAD_FN(2, 0, 1, 0, dsps)
GBHF_GRAD_FN(0, 0, 0, 0, ssss)
GBHF_GRAD_FN(0, 0, 1, 0, ssps)
GBHF_GRAD_FN(0, 0, 1, 1, sspp)
GBHF_GRAD_FN(1, 0, 0, 0, psss)
GBHF_GRAD_FN(1, 0, 1, 0, psps)
GBHF_GRAD_FN(1, 0, 1, 1, pspp)
GBHF_GRAD_FN(1, 1, 0, 0, ppss)
GBHF_GRAD_FN(1, 1, 1, 0, ppps)
GBHF_GRAD_FN(1, 1, 1, 1, pppp)

template <typename T>
struct GradArgs {
  const int4* tasks;
  const int* range;          // start, end of this class and precision
  int* counter;
  const int *pA, *pB, *pK, *poff, *kseg;
  const int4* seg;
  const T* bra;
  const T* ket;
  long long npp;
  const int* shell_f0;
  const int* shell_atom;     // global atom of each shell (grad index)
  const int* pmol;
  const int* mn;
  const long long* moff;
  const T* D;                // stacked n_m x n_m densities, this precision
  const T* boys;
  double* grad;              // 3 * natoms
  const double* sscale;      // per shell 6 component scales (d shells)
  const double* Q;           // Schwarz bound of each pair, and in FP32
  const float* Qf;
  double thr;                // drop a quartet when Q_ab Q_cd max|Gamma_abcd| is below
  float thrf;
  T jcoef;                   // weight of the Coulomb term D_ab D_cd in Gamma (0: exchange only)
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int LA, int LB, int LC, int LD, typename T, bool SG>
__global__ void __launch_bounds__(GR_THREADS) k_grad_jk(GradArgs<T> a) {
  constexpr int NA = ncart_c(LA), NB = ncart_c(LB), NC = ncart_c(LC), ND = ncart_c(LD);
  constexpr int NAB = NA * NB, NCD = NC * ND, NOUT = NAB * NCD;
  __shared__ __align__(16) T sbra[GR_WARPS][KMAX_PRIM_PAIRS * BRA_SB];
  __shared__ T sDab[GR_WARPS][NAB];
  extern __shared__ double gsm_dyn[];
  constexpr int NT = NAB * nherm_c(LC + LD);
  using GamT = typename std::conditional<SG, GamSmem<T, NOUT>, GamReg<T, NOUT>>::type;
  using TkT = typename std::conditional<SG, GamSmem<T, NT>, GamReg<T, NT>>::type;
  GamT gam;
  TkT tk;
  if constexpr (SG) {
    gam.p = reinterpret_cast<T*>(gsm_dyn) + threadIdx.x;
    tk.p = reinterpret_cast<T*>(gsm_dyn) + NOUT * GR_THREADS + threadIdx.x;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int start = a.range[0];
  const int ntask = a.range[1] - start;
  const long long npp = a.npp;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(a.counter, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntask) break;
    const int4 task = a.tasks[start + t];
    const int ib = task.x;
    // lanes beyond the task's kets split the primitive quartets (as in k_jk):
    // ket on the low lg bits of the lane, an nsb x nsk grid of bra and ket
    // primitive slices on the rest; the closing warp sum adds the slices
    const int nk = task.z;
    const int lg = 32 - __clz(max(nk, 1) - 1);
    const int nsl = 32 >> lg;
    const int slice = lane >> lg;
    const int jk = task.y + (lane & ((1 << lg) - 1));
    const int mol = a.pmol[ib];
    const int n = a.mn[mol];
    const T* __restrict__ Dm = a.D + a.moff[mol];
    const bool active = (lane & ((1 << lg) - 1)) < nk;
    const int kb0 = task.w & 0xffff, Kb = (task.w >> 16) - kb0, pb0 = a.poff[ib] + kb0;
    const int K = a.seg[a.kseg[task.y]].z;
    constexpr int KETC = sizeof(T) == 4 ? 1 : 0;   // per-ket-primitive work, as in k_jk
    int lb = 0;
    for (int l = 0, best = 1 << 30; (1 << l) <= nsl; ++l) {
      const int cost = (((Kb + (1 << l) - 1) >> l) + KETC) * ((K + (nsl >> l) - 1) / (nsl >> l));
      if (KETC ? cost < best : cost <= best) {
        best = cost;
        lb = l;
      }
    }
    const int nsb = 1 << lb, nsk = nsl >> lb;
    const int sb = slice & (nsb - 1), sk = slice >> lb;
    const unsigned rkb = (65536u + Kb - 1) / Kb;   // idx / Kb = (idx * rkb) >> 16 for idx < 16 * 36
    for (int idx = lane; idx < BRA_NFIELD * Kb; idx += 32) {
      const int f = (int)(((unsigned)idx * rkb) >> 16), k = idx - f * Kb;
      sbra[warp][k * BRA_SB + f] = a.bra[(long long)f * npp + pb0 + k];
    }
    const int A = a.pA[ib], B = a.pB[ib];
    const int a0 = a.shell_f0[A], b0 = a.shell_f0[B];
    for (int i = lane; i < NAB; i += 32) sDab[warp][i] = Dm[(long long)(a0 + i / NB) * n + b0 + i % NB];
    __syncwarp();
    T g[6] = {0, 0, 0, 0, 0, 0};
    T wgt = 0;
    if (active) {
      const int C = a.pA[jk], Dd = a.pB[jk];
      const int c0 = a.shell_f0[C], d0 = a.shell_f0[Dd];
      T gmax = T(0);
      // Gamma_abcd = jcoef D_ab D_cd - (D_ac D_bd + D_ad D_bc) / 4
#pragma unroll
      for (int ia = 0; ia < NA; ++ia)
#pragma unroll
        for (int ibb = 0; ibb < NB; ++ibb)
#pragma unroll
          for (int ic = 0; ic < NC; ++ic)
#pragma unroll
            for (int id = 0; id < ND; ++id) {
              const T dab = sDab[warp][ia * NB + ibb];
              const T dcd = Dm[(long long)(c0 + ic) * n + d0 + id];
              const T dac = Dm[(long long)(a0 + ia) * n + c0 + ic];
              const T dbd = Dm[(long long)(b0 + ibb) * n + d0 + id];
              const T dad = Dm[(long long)(a0 + ia) * n + d0 + id];
              const T dbc = Dm[(long long)(b0 + ibb) * n + c0 + ic];
              T gv = a.jcoef * dab * dcd - T(0.25) * (dac * dbd + dad * dbc);
              if constexpr (LA == 2 || LB == 2 || LC == 2 || LD == 2) {   // d components: scaled functions
                if (LA == 2) gv *= T(a.sscale[6 * A + ia]);
                if (LB == 2) gv *= T(a.sscale[6 * B + ibb]);
                if (LC == 2) gv *= T(a.sscale[6 * C + ic]);
                if (LD == 2) gv *= T(a.sscale[6 * Dd + id]);
              }
              gam.set(((ia * NB + ibb) * NC + ic) * ND + id, gv);
              gmax = fmax_t(gmax, fabs_t(gv));
            }
      // exact screening of this quartet by its own Gamma (the task lists bound it
      // by the pairs' density weights)
      bool keep;
      if constexpr (sizeof(T) == 4) keep = a.Qf[ib] * a.Qf[jk] * gmax >= a.thrf;
      else keep = a.Q[ib] * a.Q[jk] * gmax >= a.thr;
      const int4 sg = a.seg[a.kseg[jk]];
      const int len = sg.y - sg.x;
      const long long base = (long long)sg.w + (jk - sg.x);
      const int nbl = sb < Kb && keep ? (Kb - sb + nsb - 1) / nsb : 0;
      for (int kc = sk; keep && kc < K; kc += nsk) {
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
        GradFn<LA, LB, LC, LD>::ket(invq, QCx, QCy, QCz, QDx, QDy, QDz, gam, tk);
        GradFn<LA, LB, LC, LD>::run(sbra[warp] + sb * BRA_SB, nbl, nsb * BRA_SB, q, Qx, Qy, Qz, Kcd, a.boys, tk, g);
      }
      wgt = (A == B ? T(1) : T(2)) * (C == Dd ? T(1) : T(2));
    }
#pragma unroll
    for (int x = 0; x < 6; ++x) {
      T v = wgt * g[x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) atomicAdd(&a.grad[3 * a.shell_atom[x < 3 ? A : B] + x % 3], widen(v));
    }
    __syncwarp();
  }
}

template <int LA, int LB, int LC, int LD, typename T>
static gbhf_status launch_grad_class(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const T* D, const T* bra,
                                     const T* ket, const T* boys, double* grad, int ntask) {
  if (ntask <= 0) return GBHF_OK;
  constexpr int NOUT = ncart_c(LA) * ncart_c(LB) * ncart_c(LC) * ncart_c(LD);
  constexpr int NT = ncart_c(LA) * ncart_c(LB) * nherm_c(LC + LD);
  constexpr bool SG = sizeof(T) == 8 ? NOUT > 9 : NOUT > 27;   // Gamma and T in shared memory
  const size_t smem = SG ? (size_t)(NOUT + NT) * GR_THREADS * sizeof(T) : 0;
  auto kern = k_grad_jk<LA, LB, LC, LD, T, SG>;
  static bool attr_set = false;
  if (SG && !attr_set) {
    GBHF_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int per_sm = 0;
  GBHF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, GR_THREADS, smem));
  per_sm = std::max(per_sm, 1);
  const int grid = std::min(c->nsm * per_sm, (ntask + GR_WARPS - 1) / GR_WARPS);
  PairData& P = c->pairs;
  TaskLists& gt = c->gtasks;
  GradArgs<T> a;
  a.tasks = prec == 0 ? gt.tasks64.p : gt.tasks32.p;
  a.range = gt.ranges.p + 4 * combo + 2 * prec;
  a.counter = gt.counters.p + 2 * combo + prec;
  a.pA = P.A.p;
  a.pB = P.B.p;
  a.pK = P.K.p;
  a.poff = P.poff.p;
  a.kseg = P.kseg.p;
  a.seg = P.seg_info.p;
  a.bra = bra;
  a.ket = ket;
  a.npp = (long long)P.nprim_pairs;
  a.shell_f0 = c->tasks.f0.p;
  a.shell_atom = c->tasks.atom.p;
  a.pmol = P.mol.p;
  a.mn = c->tasks.mn.p;
  a.moff = c->tasks.moff.p;
  a.D = D;
  a.boys = boys;
  a.grad = grad;
  a.sscale = c->tasks.sscale.p;
  a.Q = P.Q.p;
  a.Qf = P.Qf.p;
  a.thr = gt.thr_exact;
  a.thrf = (float)gt.thr_exact;
  a.jcoef = T(c->grad_jcoef);
  kern<<<grid, GR_THREADS, smem, strm>>>(a);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

template <typename T>
static gbhf_status launch_grad_combo(gbhf_ctx* c, cudaStream_t strm, int k, int prec, const T* D, const T* bra,
                                     const T* ket, const T* boys, double* grad, int nt) {
  switch (k) {   // (bra class, ket class) = (k / 3, k % 3); class 0 = ss, 1 = ps, 2 = pp
    case 0: return launch_grad_class<0, 0, 0, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 1: return launch_grad_class<0, 0, 1, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 2: return launch_grad_class<0, 0, 1, 1, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 3: return launch_grad_class<1, 0, 0, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 4: return launch_grad_class<1, 0, 1, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 5: return launch_grad_class<1, 0, 1, 1, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 6: return launch_grad_class<1, 1, 0, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 7: return launch_grad_class<1, 1, 1, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 8: return launch_grad_class<1, 1, 1, 1, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    // combinations with a d pair on generated code (GRAD_COMBO_BRA / GRAD_COMBO_KET)
    case 9: return launch_grad_class<0, 0, 2, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 10: return launch_grad_class<0, 0, 2, 1, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 12: return launch_grad_class<1, 0, 2, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 18: return launch_grad_class<2, 0, 0, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    case 19: return launch_grad_class<2, 0, 1, 0, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
    default: return fail(c, GBHF_ERR_UNSUPPORTED, "no generated gradient kernel for combo " + std::to_string(k));
  }
}

// Gradient combinations with a d pair evaluated by the generated lane-per-ket
// code; the others go to the warp-per-quartet kernels of gradd.cu.
bool grad_gen_combo(int k) {
  return k < NGCOMBO_SP || k == 9 || k == 10 || k == 12 || k == 18 || k == 19;
}

// Two-electron gradient of D (n x n, device) into d_grad (accumulated).  With
// profiling events the launches run in order on the context stream, each timed
// into prof.gcls_ms; otherwise round-robin on the side streams.
gbhf_status grad_2e(gbhf_ctx* c, const double* d_D, double schwarz, double mixed_cutoff, int precision,
                           double* d_grad) {
  GBHF_TRY(build_grad_tasks(c, d_D, schwarz, mixed_cutoff, precision));
  TaskLists& gt = c->gtasks;
  gt.thr_exact = schwarz;   // per-quartet Gamma test in the kernels
  const size_t nst = (size_t)c->basis.stacked;
  bool any32 = false;
  for (int k = 0; k < NCOMBO_MAX; ++k) any32 |= gt.hranges[4 * k + 3] > gt.hranges[4 * k + 2];
  if (any32) {
    GBHF_CUDA(c, c->dfloat.alloc(nst));
    GBHF_TRY(to_float(c, nst, d_D, c->dfloat.p));
  }
  GBHF_CUDA(c, cudaMemsetAsync(gt.counters.p, 0, 2 * NCOMBO_MAX * sizeof(int), c->stream));
  const bool ev = c->prof.events;
  int ne = 0, ev_combo[2 * NCOMBO_MAX], ev_prec[2 * NCOMBO_MAX];
  if (ev) {
    GBHF_CUDA(c, cudaEventRecord(c->evg[0], c->stream));
  } else {
    GBHF_CUDA(c, cudaEventRecord(c->fork_ev, c->stream));
    for (int i = 0; i < gbhf_ctx::NSIDE_GRAD; ++i) GBHF_CUDA(c, cudaStreamWaitEvent(c->side[i], c->fork_ev, 0));
  }
  PairData& P = c->pairs;
  int nl = 0;
  // heaviest first: the d combinations, then the s/p ones
  static const int order[NCOMBO_MAX] = {35, 34, 29, 33, 28, 23, 32, 27, 22, 17, 31, 26, 21, 16, 11, 30, 25, 20,
                                        15, 14, 10, 24, 19, 13, 9, 18, 12, 8, 7, 5, 6, 4, 2, 3, 1, 0};
  for (int prec = 0; prec < 2; ++prec) {
    if (prec == 1 && !any32) break;
    for (int oi = 0; oi < NCOMBO_MAX; ++oi) {
      const int k = order[oi];
      const int nt = gt.hranges[4 * k + 2 * prec + 1] - gt.hranges[4 * k + 2 * prec];
      if (nt <= 0) continue;
      cudaStream_t strm = ev ? c->stream : c->side[nl++ % gbhf_ctx::NSIDE_GRAD];
      if (!grad_gen_combo(k))
        GBHF_TRY(launch_grad_dclass(c, strm, k, prec, d_D, c->dfloat.p, d_grad, nt));
      else if (prec == 0)
        GBHF_TRY(launch_grad_combo<double>(c, strm, k, 0, d_D, P.bra64.p, P.ket64.p, c->boysh64.p, d_grad, nt));
      else
        GBHF_TRY(launch_grad_combo<float>(c, strm, k, 1, c->dfloat.p, P.bra32.p, P.ket32.p, c->boysh32.p, d_grad,
                                          nt));
      if (ev) {
        ev_combo[ne] = k;
        ev_prec[ne] = prec;
        ++ne;
        GBHF_CUDA(c, cudaEventRecord(c->evg[ne], c->stream));
      }
    }
  }
  if (!ev) {
    for (int i = 0; i < gbhf_ctx::NSIDE_GRAD; ++i) {
      GBHF_CUDA(c, cudaEventRecord(c->join_ev[i], c->side[i]));
      GBHF_CUDA(c, cudaStreamWaitEvent(c->stream, c->join_ev[i], 0));
    }
    return GBHF_OK;
  }
  GBHF_CUDA(c, cudaEventSynchronize(c->evg[ne]));
  for (int e = 0; e < ne; ++e) {
    float ms = 0;
    GBHF_CUDA(c, cudaEventElapsedTime(&ms, c->evg[e], c->evg[e + 1]));
    c->prof.gcls_ms[ev_combo[e]][ev_prec[e]] += ms;
  }
  return GBHF_OK;
}

// ---------------------------------------------------------- one-electron ----
// Thread per function pair (a <= b): D-weighted derivatives of T and W-weighted
// derivatives of S (translational invariance gives d/dB = -d/dA).  Primitive
// pairs whose weighted prefactor is below 1e-17 are skipped.  The nuclear
// attraction follows in k_grad_vne.
constexpr int G1_THREADS = 64;

// Molecule-aware: row i (global function) pairs with the functions j >= i of
// its molecule; D and W are the stacked n_m x n_m blocks; the operator centres
// are the molecule's atoms.
struct Grad1eArgs {
  const double* xyz;
  const double* Z;
  const int* fn;            // per global CGF: atom (global), lx, ly, lz, np, off
  const double* coef;
  const double* expo;
  const double* tab;
  const int* fmol;          // per global CGF: molecule
  const int* mfo;           // per molecule: first function (nmol+1)
  const int* mao;           // per molecule: first atom (nmol+1)
  const long long* moff;    // per molecule: block offset in D, W
  const double* D;
  const double* W;
  double* grad;             // 3 * total atoms
};

__global__ void __launch_bounds__(G1_THREADS) k_grad_1e(Grad1eArgs g) {
  const int i = blockIdx.y;
  const int mol = g.fmol[i];
  const int f0m = g.mfo[mol], nm = g.mfo[mol + 1] - f0m;
  const int il = i - f0m;
  const int jl = blockIdx.x * blockDim.x + threadIdx.x;   // local column
  const double* __restrict__ xyz = g.xyz;
  const double* __restrict__ coef = g.coef;
  const double* __restrict__ expo = g.expo;
  double* __restrict__ grad = g.grad;
  if (jl < nm && jl >= il) {
    const int j = f0m + jl;
    const DevFn f = load_fn(g.fn, i), gfn = load_fn(g.fn, j);
    const double *A = xyz + 3 * f.atom, *B = xyz + 3 * gfn.atom;
    const double mult = (i == j) ? 1.0 : 2.0;
    const double dab = mult * g.D[g.moff[mol] + (long)il * nm + jl], wab = mult * g.W[g.moff[mol] + (long)il * nm + jl];
    double ab2 = 0;
    for (int x = 0; x < 3; ++x) ab2 += (A[x] - B[x]) * (A[x] - B[x]);
    double gA[3] = {0, 0, 0};   // d/dA of (D T - W S); d/dB = -d/dA
    for (int p1 = 0; p1 < f.np; ++p1)
      for (int p2 = 0; p2 < gfn.np; ++p2) {
        const double c1 = coef[f.off + p1], a = expo[f.off + p1];
        const double c2 = coef[gfn.off + p2], b = expo[gfn.off + p2];
        const double p = a + b, mu = a * b / p;
        const double kab = c1 * c2 * exp(-mu * ab2);
        if (fabs(kab) * (1.0 + p) * (fabs(dab) * (1.0 + p) + fabs(wab)) * (GBHF_PI / p) * sqrt(GBHF_PI / p) < 1e-17)
          continue;
        const double cte = sqrt(GBHF_PI / p);
        double P[3], s[3][4][5];   // up to l_a + 1 <= 3 on A, l_b + 2 <= 4 on B
        for (int x = 0; x < 3; ++x) {
          P[x] = (a * A[x] + b * B[x]) / p;
          const double abx = A[x] - B[x];
          // table up to i+1 on A and j+2 on B (kinetic)
          const double s00 = exp(-mu * abx * abx) * cte;
          const double c = 1.0 / (2.0 * p);
          const double pax = P[x] - A[x], pbx = P[x] - B[x];
          for (int m = 0; m <= f.l[x] + 1; ++m)
            for (int nn = 0; nn <= gfn.l[x] + 2; ++nn) {
              double v;
              if (m == 0 && nn == 0) v = s00;
              else if (m == 0) v = pbx * s[x][0][nn - 1] + (nn >= 2 ? c * (nn - 1) * s[x][0][nn - 2] : 0.0);
              else if (nn == 0) v = pax * s[x][m - 1][0] + (m >= 2 ? c * (m - 1) * s[x][m - 2][0] : 0.0);
              else v = pax * s[x][m - 1][nn] + c * ((m >= 2 ? (m - 1) * s[x][m - 2][nn] : 0.0) + nn * s[x][m - 1][nn - 1]);
              s[x][m][nn] = v;
            }
        }
        auto S1 = [&](int x, int m, int nn) { return (m < 0 || nn < 0) ? 0.0 : s[x][m][nn]; };
        auto T1 = [&](int x, int m, int nn) {   // kinetic 1-D term
          if (m < 0) return 0.0;
          return -2.0 * b * b * S1(x, m, nn + 2) + b * (2 * nn + 1) * S1(x, m, nn) -
                 (nn >= 2 ? 0.5 * nn * (nn - 1) * S1(x, m, nn - 2) : 0.0);
        };
        double sx[3], tx[3], dsx[3], dtx[3];
        for (int x = 0; x < 3; ++x) {
          const int li = f.l[x], lj = gfn.l[x];
          sx[x] = S1(x, li, lj);
          tx[x] = T1(x, li, lj);
          dsx[x] = 2 * a * S1(x, li + 1, lj) - li * S1(x, li - 1, lj);
          dtx[x] = 2 * a * T1(x, li + 1, lj) - li * T1(x, li - 1, lj);
        }
        for (int dir = 0; dir < 3; ++dir) {
          // d/dA_dir of S and T: the axis-dir factor becomes 2a f(i+1) - i f(i-1)
          double dS = 1.0, dT = 0;
          for (int x = 0; x < 3; ++x) dS *= (x == dir) ? dsx[x] : sx[x];
          for (int k = 0; k < 3; ++k) {
            double term = 1.0;
            for (int x = 0; x < 3; ++x) {
              if (x == k) term *= (x == dir) ? dtx[x] : tx[x];
              else term *= (x == dir) ? dsx[x] : sx[x];
            }
            dT += term;
          }
          gA[dir] += c1 * c2 * (dab * dT - wab * dS);
        }
      }
    for (int x = 0; x < 3; ++x) {
      atomicAdd(&grad[3 * f.atom + x], gA[x]);
      atomicAdd(&grad[3 * gfn.atom + x], -gA[x]);
    }
  }
}

// Nuclear-attraction terms: warp per shell pair of class (LA, LB), lanes over the
// molecule's nuclei; generated per-primitive-pair code (grad_gen.cuh).  The pair
// covers (a, b) and (b, a) when A != B (weight 2).  Bra-centre sums are reduced
// over the warp; each lane adds the operator-centre term -(dA + dB) of its nucleus.
template <int LA, int LB>
struct VneFn;
template <>
struct VneFn<0, 0> {
  static __device__ __forceinline__ void run(const BraPrim<double>& bp, double x, double y, double z, double zp,
                                             const double* dw, const double* boys, double* g) {
    vne_grad_ss<double>(bp, x, y, z, zp, dw, boys, g);
  }
};
template <>
struct VneFn<1, 0> {
  static __device__ __forceinline__ void run(const BraPrim<double>& bp, double x, double y, double z, double zp,
                                             const double* dw, const double* boys, double* g) {
    vne_grad_ps<double>(bp, x, y, z, zp, dw, boys, g);
  }
};
template <>
struct VneFn<1, 1> {
  static __device__ __forceinline__ void run(const BraPrim<double>& bp, double x, double y, double z, double zp,
                                             const double* dw, const double* boys, double* g) {
    vne_grad_pp<double>(bp, x, y, z, zp, dw, boys, g);
  }
};
template <>
struct VneFn<2, 0> {
  static __device__ __forceinline__ void run(const BraPrim<double>& bp, double x, double y, double z, double zp,
                                             const double* dw, const double* boys, double* g) {
    vne_grad_ds<double>(bp, x, y, z, zp, dw, boys, g);
  }
};
template <>
struct VneFn<2, 1> {
  static __device__ __forceinline__ void run(const BraPrim<double>& bp, double x, double y, double z, double zp,
                                             const double* dw, const double* boys, double* g) {
    vne_grad_dp<double>(bp, x, y, z, zp, dw, boys, g);
  }
};
template <>
struct VneFn<2, 2> {
  static __device__ __forceinline__ void run(const BraPrim<double>& bp, double x, double y, double z, double zp,
                                             const double* dw, const double* boys, double* g) {
    vne_grad_dd<double>(bp, x, y, z, zp, dw, boys, g);
  }
};

struct VneArgs {
  int p0, p1;               // pairs of this class
  const int *pA, *pB, *pK, *poff, *pmol;
  const double* bra;        // pair-contiguous primitive-pair fields
  long long npp;
  const int* shell_f0;      // within the molecule
  const int* shell_atom;
  const double* sscale;     // per shell 6 component scales (d shells)
  const int* mn;
  const long long* moff;
  const int* mao;           // first atom of each molecule (nmol + 1)
  const double* xyz;
  const double* Z;
  const double* D;          // stacked
  const double* boys;       // FP64 Horner tables
  double kvf;               // 2 pi / sqrt(2 pi^2.5): K' of the pair data -> 2 pi/p c c exp(-mu AB^2)
  double* grad;
};

template <int LA, int LB>
__global__ void __launch_bounds__(128) k_grad_vne(VneArgs a) {
  constexpr int NA = ncart_c(LA), NB = ncart_c(LB);
  const int lane = threadIdx.x & 31;
  const int pr = a.p0 + blockIdx.x * 4 + (threadIdx.x >> 5);
  if (pr >= a.p1) return;
  const int A = a.pA[pr], B = a.pB[pr], mol = a.pmol[pr], n = a.mn[mol];
  const double* Dm = a.D + a.moff[mol];
  const int fa = a.shell_f0[A], fb = a.shell_f0[B];
  const double mult = A == B ? 1.0 : 2.0;
  double dw[NA * NB];
  double dmax = 0;
#pragma unroll
  for (int ia = 0; ia < NA; ++ia)
#pragma unroll
    for (int ib = 0; ib < NB; ++ib) {
      dw[ia * NB + ib] = mult * Dm[(long)(fa + ia) * n + fb + ib] * a.sscale[6 * A + ia] * a.sscale[6 * B + ib];
      dmax = fmax(dmax, fabs(dw[ia * NB + ib]));
    }
  double gAB[6] = {0, 0, 0, 0, 0, 0};
  const int K = a.pK[pr];
  const long long po = a.poff[pr];
  const int c0 = a.mao[mol], c1 = a.mao[mol + 1];
  for (int cb = c0; cb < c1; cb += 32) {
    const int cn = cb + lane;
    if (cn < c1) {
      const double Cx = a.xyz[3 * cn], Cy = a.xyz[3 * cn + 1], Cz = a.xyz[3 * cn + 2], Zc = a.Z[cn];
      double gC[3] = {0, 0, 0};
      for (int k = 0; k < K; ++k) {
        BraPrim<double> bp;
        const long long idx = po + k;
        bp.p = a.bra[BRA_P * a.npp + idx];
        bp.invp = a.bra[BRA_INVP * a.npp + idx];
        bp.Px = a.bra[BRA_PX * a.npp + idx];
        bp.Py = a.bra[BRA_PY * a.npp + idx];
        bp.Pz = a.bra[BRA_PZ * a.npp + idx];
        bp.PAx = a.bra[BRA_PAX * a.npp + idx];
        bp.PAy = a.bra[BRA_PAY * a.npp + idx];
        bp.PAz = a.bra[BRA_PAZ * a.npp + idx];
        bp.PBx = a.bra[BRA_PBX * a.npp + idx];
        bp.PBy = a.bra[BRA_PBY * a.npp + idx];
        bp.PBz = a.bra[BRA_PBZ * a.npp + idx];
        bp.K = a.bra[BRA_K * a.npp + idx];
        bp.a = a.bra[BRA_AEXP * a.npp + idx];
        const double zpref = -Zc * bp.K * a.kvf;
        if (fabs(zpref) * dmax * (1.0 + bp.p) < 1e-17) continue;
        double g6[6] = {0, 0, 0, 0, 0, 0};
        VneFn<LA, LB>::run(bp, Cx, Cy, Cz, zpref, dw, a.boys, g6);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          gAB[x] += g6[x];
          gAB[3 + x] += g6[3 + x];
          gC[x] -= g6[x] + g6[3 + x];
        }
      }
#pragma unroll
      for (int x = 0; x < 3; ++x)
        if (gC[x] != 0.0) atomicAdd(&a.grad[3 * cn + x], gC[x]);
    }
  }
#pragma unroll
  for (int x = 0; x < 6; ++x) {
    const double v = warp_sum_d(gAB[x]);
    if (lane == 0 && v != 0.0) atomicAdd(&a.grad[3 * a.shell_atom[x < 3 ? A : B] + x % 3], v);
  }
}

template <int LA, int LB>
static gbhf_status launch_vne(gbhf_ctx* c, int cls, const double* d_D, double* d_grad) {
  PairData& P = c->pairs;
  VneArgs a;
  a.p0 = P.cls_start[cls];
  a.p1 = P.cls_start[cls + 1];
  if (a.p1 <= a.p0) return GBHF_OK;
  a.pA = P.A.p;
  a.pB = P.B.p;
  a.pK = P.K.p;
  a.poff = P.poff.p;
  a.pmol = P.mol.p;
  a.bra = P.bra64.p;
  a.npp = (long long)P.nprim_pairs;
  a.shell_f0 = c->tasks.f0.p;
  a.shell_atom = c->tasks.atom.p;
  a.sscale = c->tasks.sscale.p;
  a.mn = c->tasks.mn.p;
  a.moff = c->tasks.moff.p;
  a.mao = c->tasks.mao.p;
  a.xyz = c->d_xyz.p;
  a.Z = c->d_Z.p;
  a.D = d_D;
  a.boys = c->boysh64.p;
  a.kvf = 2.0 * GBHF_PI / std::sqrt(TWO_PI_2P5);
  a.grad = d_grad;
  k_grad_vne<LA, LB><<<(a.p1 - a.p0 + 3) / 4, 128, 0, c->stream>>>(a);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// Nuclear repulsion gradient, one thread per atom: -sum_L Z_K Z_L (R_K - R_L) / R_KL^3
// over the atoms L of the same molecule.
__global__ void k_grad_nuc(int natoms, const int* __restrict__ amol, const int* __restrict__ mao,
                           const double* __restrict__ xyz, const double* __restrict__ Z, double* __restrict__ grad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= natoms) return;
  const int m = amol[k];
  double g[3] = {0, 0, 0};
  for (int l = mao[m]; l < mao[m + 1]; ++l) {
    if (l == k) continue;
    double d[3], r2 = 0;
    for (int x = 0; x < 3; ++x) {
      d[x] = xyz[3 * k + x] - xyz[3 * l + x];
      r2 += d[x] * d[x];
    }
    const double f = Z[k] * Z[l] / (r2 * sqrt(r2));
    for (int x = 0; x < 3; ++x) g[x] -= f * d[x];
  }
  for (int x = 0; x < 3; ++x) grad[3 * k + x] += g[x];
}

// Host driver: D and W square (device), gradient into d_grad (3*natoms, device).
gbhf_status gradient_dev(gbhf_ctx* c, const double* d_D, const double* d_W, double schwarz, double mixed_cutoff,
                         int precision, double* d_grad) {
  const Basis& b = c->basis;
  if (!b.shells_ok || b.maxL > 2)
    return fail(c, GBHF_ERR_UNSUPPORTED, "gradient kernels need complete s, p and d shells");
  GBHF_TRY(ensure_boys_tables(c));
  GBHF_TRY(ensure_pairs(c));
  const int n = b.nbf, na = b.natoms;
  GBHF_TRY(ensure_shell_arrays(c));
  GBHF_CUDA(c, cudaMemsetAsync(d_grad, 0, 3 * na * sizeof(double), c->stream));
  k_grad_nuc<<<(na + 127) / 128, 128, 0, c->stream>>>(na, c->tasks.amol.p, c->tasks.mao.p, c->d_xyz.p, c->d_Z.p,
                                                      d_grad);
  int max_fn = 0;
  for (int m = 0; m < b.nmol; ++m) max_fn = std::max(max_fn, b.mol_fn_off[m + 1] - b.mol_fn_off[m]);
  Grad1eArgs g1;
  g1.xyz = c->d_xyz.p;
  g1.Z = c->d_Z.p;
  g1.fn = c->d_fn.p;
  g1.coef = c->d_coef.p;
  g1.expo = c->d_exp.p;
  g1.tab = c->boys64.p;
  g1.fmol = c->tasks.fmol.p;
  g1.mfo = c->tasks.mfo.p;
  g1.mao = c->tasks.mao.p;
  g1.moff = c->tasks.moff.p;
  g1.D = d_D;
  g1.W = d_W;
  g1.grad = d_grad;
  k_grad_1e<<<dim3((max_fn + G1_THREADS - 1) / G1_THREADS, n), G1_THREADS, 0, c->stream>>>(g1);
  count_launch(c, 2);
  GBHF_CUDA(c, cudaGetLastError());
  GBHF_TRY((launch_vne<0, 0>(c, 0, d_D, d_grad)));
  GBHF_TRY((launch_vne<1, 0>(c, 1, d_D, d_grad)));
  GBHF_TRY((launch_vne<1, 1>(c, 2, d_D, d_grad)));
  GBHF_TRY((launch_vne<2, 0>(c, 3, d_D, d_grad)));
  GBHF_TRY((launch_vne<2, 1>(c, 4, d_D, d_grad)));
  GBHF_TRY((launch_vne<2, 2>(c, 5, d_D, d_grad)));
  GBHF_TRY(grad_2e(c, d_D, schwarz, mixed_cutoff, precision, d_grad));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

// W = 2 sum_{i < nocc} eps_i C_i C_i^T  (energy-weighted density)
__global__ void k_scale_occ(int n, int nocc, const double* __restrict__ C, const double* __restrict__ eps,
                            double* __restrict__ out) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nocc) return;
  out[(long)i * nocc + j] = C[(long)i * n + j] * eps[j];
}

// UHF gradient: D_a, D_b and W square (device), gradient into d_grad.
gbhf_status gradient_uhf_dev(gbhf_ctx* c, const double* d_Da, const double* d_Db, const double* d_W, double schwarz,
                             double mixed_cutoff, int precision, double* d_grad) {
  const size_t nn = (size_t)c->basis.nbf * c->basis.nbf;
  DBuf<double> DT, DS;
  GBHF_CUDA(c, DT.alloc(nn));
  GBHF_CUDA(c, DS.alloc(nn));
  GBHF_TRY(axpby(c, nn, 1.0, d_Da, 1.0, d_Db, DT.p));
  GBHF_TRY(axpby(c, nn, 1.0, d_Da, -1.0, d_Db, DS.p));
  GBHF_TRY(gradient_dev(c, DT.p, d_W, schwarz, mixed_cutoff, precision, d_grad));
  c->grad_jcoef = 0.0;
  const gbhf_status st = grad_2e(c, DS.p, schwarz, mixed_cutoff, precision, d_grad);
  c->grad_jcoef = 1.0;
  GBHF_TRY(st);
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

gbhf_status energy_weighted_density(gbhf_ctx* c, int n, int nocc, const double* d_C, const double* d_eps,
                                    double* d_W) {
  if (nocc <= 0) {
    GBHF_CUDA(c, cudaMemsetAsync(d_W, 0, (size_t)n * n * sizeof(double), c->stream));
    return GBHF_OK;
  }
  GBHF_WS(c, T, 23, (size_t)n * nocc);
  k_scale_occ<<<dim3((nocc + 127) / 128, n), 128, 0, c->stream>>>(n, nocc, d_C, d_eps, T);
  count_launch(c);
  // W = 2 (C eps)_occ C_occ^T with C_occ the first nocc columns of C (ldb = n)
  GBHF_TRY(gemm(c, false, true, n, n, nocc, 2.0, T, nocc, d_C, n, 0.0, d_W, n));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

}  // namespace gbhf
