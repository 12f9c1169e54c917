// Two-electron gradient for the (bra class, ket class) combinations that hold
// a d shell: one warp per contracted shell quartet (mdwarp.cuh), bra-centre
// derivatives only, as the s/p kernels of grad.cu.  Summed over every ordered
// pair of shell pairs with weights (2 - delta_AB)(2 - delta_CD), the
// bra-centre terms give the whole two-electron gradient.
//
// Per quartet the warp forms Gamma_abcd = jcoef D_ab D_cd - (D_ac D_bd + D_ad D_bc)/4
// (with the pair weights and the d-component scales) in shared memory; per
// primitive quartet it builds X[h][cd] for the bra Hermite range one order up
// and contracts Z[ab][h] = sum_cd Gamma_abcd X[h][cd] with the derivative
// Hermite coefficients dE^ab_h/dA = 2a E^(a+1,b)_h - a_x E^(a-1,b)_h
// (and the same in b for B).
#include <algorithm>
#include <string>

#include "gbhf_internal.h"
#include "mdwarp.cuh"

namespace gbhf {

constexpr int GRD_WARPS = 2;
constexpr int GRD_THREADS = 32 * GRD_WARPS;
constexpr int GRD_TUV_BYTES = ((nherm(BOYSH_LMAX) * 4 + 15) / 16) * 16;

template <typename T>
struct GradDArgs {
  const int4* tasks;
  const int* range;
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
  const int* shell_atom;
  const int* pmol;
  const int* mn;
  const long long* moff;
  const double* sscale;
  const T* D;
  const T* boys;
  const double* Q;       // Schwarz bound of each pair
  double thr;            // drop a quartet when Q_ab Q_cd max|Gamma_abcd| is below
  double* grad;
  T jcoef;               // weight of the Coulomb term D_ab D_cd in Gamma (0: exchange only)
};

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(GRD_THREADS) k_gradd(GradDArgs<T> a) {
  using C = MDCfg<LA, LB, LC, LD, 1>;
  extern __shared__ __align__(16) unsigned char grd_smem[];
  int* tuv = reinterpret_cast<int*>(grd_smem);
  md_fill_tuv(tuv, C::L);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* ws = reinterpret_cast<T*>(grd_smem + GRD_TUV_BYTES) + warp * C::WS;
  T* sbra = ws + C::OFF_SB;
  T* Gam = ws + C::OFF_G;
  const int start = a.range[0], ntask = a.range[1] - start;
  const long long npp = a.npp;
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
    const int kb0 = task.w & 0xffff, Kb = (task.w >> 16) - kb0, pb0 = a.poff[ib] + kb0;
    const unsigned rkb = (65536u + Kb - 1) / Kb;   // idx / Kb = (idx * rkb) >> 16 for idx < 16 * 36
    for (int idx = lane; idx < BRA_NFIELD * Kb; idx += 32) {
      const int f = (int)(((unsigned)idx * rkb) >> 16), k = idx - f * Kb;
      sbra[k * BRA_SB + f] = a.bra[(long long)f * npp + pb0 + k];
    }
    const int A = a.pA[ib], B = a.pB[ib];
    const int a0 = a.shell_f0[A], b0 = a.shell_f0[B];
    T g[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    for (int q = 0; q < task.z; ++q) {
      const int jk = task.y + q;
      const int Cs = a.pA[jk], Ds = a.pB[jk];
      const int c0 = a.shell_f0[Cs], d0 = a.shell_f0[Ds];
      const T wgt = (A == B ? T(1) : T(2)) * (Cs == Ds ? T(1) : T(2));
      double gmax = 0.0;
      for (int e = lane; e < C::NOUT; e += 32) {
        const int ab = e / C::NCD, cd = e - ab * C::NCD;
        const int ia = ab / C::NB, ibb = ab - ia * C::NB, ic = cd / C::ND, id = cd - ic * C::ND;
        const T dab = Dm[(long long)(a0 + ia) * n + b0 + ibb], dcd = Dm[(long long)(c0 + ic) * n + d0 + id];
        const T dac = Dm[(long long)(a0 + ia) * n + c0 + ic], dbd = Dm[(long long)(b0 + ibb) * n + d0 + id];
        const T dad = Dm[(long long)(a0 + ia) * n + d0 + id], dbc = Dm[(long long)(b0 + ibb) * n + c0 + ic];
        const double sc = a.sscale[6 * A + ia] * a.sscale[6 * B + ibb] * a.sscale[6 * Cs + ic] * a.sscale[6 * Ds + id];
        const T gv = (a.jcoef * dab * dcd - T(0.25) * (dac * dbd + dad * dbc)) * T(sc);
        Gam[e] = gv * wgt;
        gmax = fmax(gmax, fabs((double)gv));
      }
      __syncwarp();
      // exact screening of this quartet by its own Gamma (warp-uniform decision)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) gmax = fmax(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
      if (a.Q[ib] * a.Q[jk] * gmax < a.thr) continue;
      const int4 sg = a.seg[a.kseg[jk]];
      const int K = sg.z, len = sg.y - sg.x;
      const long long base = (long long)sg.w + (jk - sg.x);
      for (int kb = 0; kb < Kb; ++kb) {
        MDPrim<T> bp;
        md_row_prim(sbra + kb * BRA_SB, bp);
        const T ea = sbra[kb * BRA_SB + BRA_AEXP], eb = bp.p - ea;
        md_bra_e<C>(ws, bp, lane);
        for (int kc = 0; kc < K; ++kc) {
          MDPrim<T> kp;
          md_load_prim(a.ket, npp, base + (long long)kc * len, kp);
          md_prim_x<C>(ws, tuv, bp, kp, a.boys, lane);
          md_bra_grad<C>(ws, tuv, ea, eb, g, lane);
          __syncwarp();
        }
      }
    }
#pragma unroll
    for (int x = 0; x < 6; ++x) {
      T v = g[x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) atomicAdd(&a.grad[3 * a.shell_atom[x < 3 ? A : B] + x % 3], widen(v));
    }
    __syncwarp();
  }
}

template <int LA, int LB, int LC, int LD, typename T>
static gbhf_status launch_gradd_t(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const T* D, const T* bra,
                                  const T* ket, const T* boys, double* grad, int ntask) {
  if (ntask <= 0) return GBHF_OK;
  using C = MDCfg<LA, LB, LC, LD, 1>;
  const size_t smem = GRD_TUV_BYTES + (size_t)GRD_WARPS * C::WS * sizeof(T);
  auto kern = k_gradd<LA, LB, LC, LD, T>;
  static bool attr_set = false;
  if (!attr_set) {
    GBHF_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int per_sm = 0;
  GBHF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, GRD_THREADS, smem));
  per_sm = std::max(per_sm, 1);
  const int grid = std::min(c->nsm * per_sm, (ntask + GRD_WARPS - 1) / GRD_WARPS);
  PairData& P = c->pairs;
  TaskLists& gt = c->gtasks;
  GradDArgs<T> a;
  a.tasks = prec == 0 ? gt.tasks64.p : gt.tasks32.p;
  a.range = gt.ranges.p + 4 * combo + 2 * prec;
  a.counter = gt.counters.p + 2 * combo + prec;
  a.pA = P.A.p;
  a.pB = P.B.p;
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
  a.sscale = c->tasks.sscale.p;
  a.Q = P.Q.p;
  a.thr = gt.thr_exact;
  a.jcoef = T(c->grad_jcoef);
  a.D = D;
  a.boys = boys;
  a.grad = grad;
  kern<<<grid, GRD_THREADS, smem, strm>>>(a);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  return GBHF_OK;
}

// Gradient combos 9..35: every ordered (bra class, ket class) with a d pair
// class (3 = ds, 4 = dp, 5 = dd), in GRAD_COMBO_BRA / GRAD_COMBO_KET order.
template <typename T>
static gbhf_status launch_gradd_combo(gbhf_ctx* c, cudaStream_t strm, int k, int prec, const T* D, const T* bra,
                                      const T* ket, const T* boys, double* grad, int nt) {
#define GBHF_GRD(K, la, lb, lc, ld) \
  case K: return launch_gradd_t<la, lb, lc, ld, T>(c, strm, k, prec, D, bra, ket, boys, grad, nt);
  switch (k) {
    GBHF_GRD(9, 0, 0, 2, 0)
    GBHF_GRD(10, 0, 0, 2, 1)
    GBHF_GRD(11, 0, 0, 2, 2)
    GBHF_GRD(12, 1, 0, 2, 0)
    GBHF_GRD(13, 1, 0, 2, 1)
    GBHF_GRD(14, 1, 0, 2, 2)
    GBHF_GRD(15, 1, 1, 2, 0)
    GBHF_GRD(16, 1, 1, 2, 1)
    GBHF_GRD(17, 1, 1, 2, 2)
    GBHF_GRD(18, 2, 0, 0, 0)
    GBHF_GRD(19, 2, 0, 1, 0)
    GBHF_GRD(20, 2, 0, 1, 1)
    GBHF_GRD(21, 2, 0, 2, 0)
    GBHF_GRD(22, 2, 0, 2, 1)
    GBHF_GRD(23, 2, 0, 2, 2)
    GBHF_GRD(24, 2, 1, 0, 0)
    GBHF_GRD(25, 2, 1, 1, 0)
    GBHF_GRD(26, 2, 1, 1, 1)
    GBHF_GRD(27, 2, 1, 2, 0)
    GBHF_GRD(28, 2, 1, 2, 1)
    GBHF_GRD(29, 2, 1, 2, 2)
    GBHF_GRD(30, 2, 2, 0, 0)
    GBHF_GRD(31, 2, 2, 1, 0)
    GBHF_GRD(32, 2, 2, 1, 1)
    GBHF_GRD(33, 2, 2, 2, 0)
    GBHF_GRD(34, 2, 2, 2, 1)
    GBHF_GRD(35, 2, 2, 2, 2)
    default: return fail(c, GBHF_ERR_UNSUPPORTED, "no d-class gradient kernel for combo " + std::to_string(k));
  }
#undef GBHF_GRD
}

gbhf_status launch_grad_dclass(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const double* D64,
                               const float* D32, double* grad, int ntask) {
  PairData& P = c->pairs;
  if (prec == 0)
    return launch_gradd_combo<double>(c, strm, combo, 0, D64, P.bra64.p, P.ket64.p, c->boysh64.p, grad, ntask);
  return launch_gradd_combo<float>(c, strm, combo, 1, D32, P.bra32.p, P.ket32.p, c->boysh32.p, grad, ntask);
}

}  // namespace gbhf
