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
#include <algorithm>
#include <cmath>
#include <vector>

#include "gbhf_internal.h"
#include "gbhf_md.cuh"

namespace gbhf {

namespace {

constexpr int GL = 6;          // R table dimension (L + 1 <= 5 for s, p quartets)

// Hermite E per axis with i <= IA, j <= IB, t <= i + j; E^00_0 = 1.
template <int IA, int IB>
struct EAxT {
  double v[IA + 1][IB + 1][IA + IB + 1];
  __device__ __forceinline__ double get(int i, int j, int t) const {
    if (i < 0 || j < 0 || t < 0 || t > i + j) return 0.0;
    return v[i][j][t];
  }
  __device__ __forceinline__ void build(double hp, double pa, double pb) {
#pragma unroll
    for (int i = 0; i <= IA; ++i)
#pragma unroll
      for (int j = 0; j <= IB; ++j)
#pragma unroll
        for (int t = 0; t <= i + j; ++t) {
          double val;
          if (i == 0 && j == 0 && t == 0) val = 1.0;
          else if (t == 0 && i >= 1) val = pa * get(i - 1, j, 0) + get(i - 1, j, 1);
          else if (t == 0) val = pb * get(i, j - 1, 0) + get(i, j - 1, 1);
          else val = (hp / t) * (i * get(i - 1, j, t - 1) + j * get(i, j - 1, t - 1));
          v[i][j][t] = val;
        }
  }
};

__device__ __forceinline__ void comp_of(int L, int c, int* l) {
  l[0] = l[1] = l[2] = 0;
  if (L == 1) l[c] = 1;
}

// R^0_tuv up to total order L, stored R[t][u][v] with dims GL.
__device__ void r_table(int L, double alpha, double X, double Y, double Z, const double* F, double* R) {
  hermite_r<GL - 1>(L, alpha, X, Y, Z, F, R);
}

}  // namespace

// Bra-side derivative contributions of one shell quartet (AB|CD):
// gA[3], gB[3] += 4 s sum_prims sum_abcd Gamma_abcd d(ab|cd)/dA,B.
template <int LA, int LB, int LC, int LD>
__device__ void quartet_bra_grad(const double* RA, const double* RB, const double* RC, const double* RD,
                                 const double* ea, const double* ca, int na_p, const double* eb, const double* cb,
                                 int nb_p, const double* ec, const double* cc, int nc_p, const double* ed,
                                 const double* cd, int nd_p, const double* Gamma, const double* tab, double wgt,
                                 double* gA, double* gB) {
  constexpr int NA = (LA + 1) * (LA + 2) / 2, NB = (LB + 1) * (LB + 2) / 2;
  constexpr int NC = (LC + 1) * (LC + 2) / 2, ND = (LD + 1) * (LD + 2) / 2;
  constexpr int L = LA + LB + LC + LD + 1;       // one order higher for the derivative
  constexpr int HB = LA + LB + 1;                  // bra Hermite range (derivative)
  double F[GL + 1];
  double R[GL * GL * GL];
  double ab2 = 0, cd2 = 0;
  for (int x = 0; x < 3; ++x) {
    ab2 += (RA[x] - RB[x]) * (RA[x] - RB[x]);
    cd2 += (RC[x] - RD[x]) * (RC[x] - RD[x]);
  }
  for (int ia = 0; ia < na_p; ++ia)
    for (int ib = 0; ib < nb_p; ++ib) {
      const double a = ea[ia], b = eb[ib], p = a + b;
      const double Kab = ca[ia] * cb[ib] * exp(-a * b / p * ab2);
      double P[3];
      EAxT<LA + 1, LB + 1> Eb[3];
      for (int x = 0; x < 3; ++x) {
        P[x] = (a * RA[x] + b * RB[x]) / p;
        Eb[x].build(0.5 / p, P[x] - RA[x], P[x] - RB[x]);
      }
      for (int ic = 0; ic < nc_p; ++ic)
        for (int id = 0; id < nd_p; ++id) {
          const double c = ec[ic], d = ed[id], q = c + d;
          const double Kcd = cc[ic] * cd[id] * exp(-c * d / q * cd2);
          double Q[3];
          EAxT<LC, LD> Ek[3];
          for (int x = 0; x < 3; ++x) {
            Q[x] = (c * RC[x] + d * RD[x]) / q;
            Ek[x].build(0.5 / q, Q[x] - RC[x], Q[x] - RD[x]);
          }
          const double alpha = p * q / (p + q);
          const double X = P[0] - Q[0], Y = P[1] - Q[1], Z = P[2] - Q[2];
          boys_generic(false, nullptr, tab, L, alpha * (X * X + Y * Y + Z * Z), F);
          r_table(L, alpha, X, Y, Z, F, R);
          const double pref = wgt * 4.0 * 34.98683665524972 / (p * q * sqrt(p + q)) * Kab * Kcd;
          // Y^{ab}_{tuv} = sum_cd Gamma_abcd W^{cd}_{tuv},  W^{cd}_{tuv} = sum (-1)^.. E^cd R
          for (int ka = 0; ka < NA; ++ka)
            for (int kb = 0; kb < NB; ++kb) {
              int la[3], lb[3];
              comp_of(LA, ka, la);
              comp_of(LB, kb, lb);
              // derivative bra Hermite range per axis: t <= la+lb+1
              double Yv[HB + 1][HB + 1][HB + 1];
              for (int t = 0; t <= HB; ++t)
                for (int u = 0; u <= HB; ++u)
                  for (int v = 0; v <= HB; ++v) Yv[t][u][v] = 0.0;
              for (int kc = 0; kc < NC; ++kc)
                for (int kd = 0; kd < ND; ++kd) {
                  const double g = Gamma[((ka * NB + kb) * NC + kc) * ND + kd];
                  if (g == 0.0) continue;
                  int lc[3], ld[3];
                  comp_of(LC, kc, lc);
                  comp_of(LD, kd, ld);
                  for (int t = 0; t <= la[0] + lb[0] + 1; ++t)
                    for (int u = 0; u <= la[1] + lb[1] + 1; ++u)
                      for (int v = 0; v <= la[2] + lb[2] + 1; ++v) {
                        if (t + u + v > HB) continue;
                        double w = 0;
                        for (int tau = 0; tau <= lc[0] + ld[0]; ++tau)
                          for (int nu = 0; nu <= lc[1] + ld[1]; ++nu)
                            for (int phi = 0; phi <= lc[2] + ld[2]; ++phi) {
                              const double e = Ek[0].get(lc[0], ld[0], tau) * Ek[1].get(lc[1], ld[1], nu) *
                                               Ek[2].get(lc[2], ld[2], phi);
                              const double r = R[((t + tau) * GL + (u + nu)) * GL + (v + phi)];
                              w += ((tau + nu + phi) & 1) ? -e * r : e * r;
                            }
                        Yv[t][u][v] += g * w;
                      }
                }
              // contract with differentiated bra E for the 3 axes of A and B
              for (int dir = 0; dir < 3; ++dir) {
                double sA = 0, sB = 0;
                for (int t = 0; t <= la[0] + lb[0] + 1; ++t)
                  for (int u = 0; u <= la[1] + lb[1] + 1; ++u)
                    for (int v = 0; v <= la[2] + lb[2] + 1; ++v) {
                      if (t + u + v > HB) continue;
                      const int tt[3] = {t, u, v};
                      double eA = 1, eB = 1;
                      for (int x = 0; x < 3; ++x) {
                        const int i = la[x], j = lb[x];
                        if (x == dir) {
                          eA *= 2 * a * Eb[x].get(i + 1, j, tt[x]) - i * Eb[x].get(i - 1, j, tt[x]);
                          eB *= 2 * b * Eb[x].get(i, j + 1, tt[x]) - j * Eb[x].get(i, j - 1, tt[x]);
                        } else {
                          const double e = Eb[x].get(i, j, tt[x]);
                          eA *= e;
                          eB *= e;
                        }
                      }
                      sA += eA * Yv[t][u][v];
                      sB += eB * Yv[t][u][v];
                    }
                gA[dir] += pref * sA;
                gB[dir] += pref * sB;
              }
            }
        }
    }
}

struct GradShell {
  int atom, L, np, f0;
  int off;   // primitive offset into exps/coefs
};

struct GradArgs {
  int nq;
  const int4* quartets;      // (A, B, C, D) shells with A>=B pair ordering irrelevant
  const double* qweight;     // degeneracy weight s per quartet
  const GradShell* sh;
  const double* exps;
  const double* coefs;
  const double* xyz;
  const double* D;           // n x n
  int n;
  const double* tab;
  double* grad;              // 3 * natoms
};

template <int LA, int LB, int LC, int LD>
__device__ void quartet_grad(const GradArgs& g, int4 q, double wgt) {
  constexpr int NA = (LA + 1) * (LA + 2) / 2, NB = (LB + 1) * (LB + 2) / 2;
  constexpr int NC = (LC + 1) * (LC + 2) / 2, ND = (LD + 1) * (LD + 2) / 2;
  const GradShell &A = g.sh[q.x], &B = g.sh[q.y], &C = g.sh[q.z], &Dd = g.sh[q.w];
  const int n = g.n;
  double Gam[NA * NB * NC * ND];
  double GamT[NC * ND * NA * NB];
  for (int a = 0; a < NA; ++a)
    for (int b = 0; b < NB; ++b)
      for (int c = 0; c < NC; ++c)
        for (int d = 0; d < ND; ++d) {
          const int fa = A.f0 + a, fb = B.f0 + b, fc = C.f0 + c, fd = Dd.f0 + d;
          const double val = g.D[(long)fa * n + fb] * g.D[(long)fc * n + fd] -
                             0.25 * (g.D[(long)fa * n + fc] * g.D[(long)fb * n + fd] +
                                     g.D[(long)fa * n + fd] * g.D[(long)fb * n + fc]);
          Gam[((a * NB + b) * NC + c) * ND + d] = val;
          GamT[((c * ND + d) * NA + a) * NB + b] = val;
        }
  double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0}, gD[3] = {0, 0, 0};
  const double *RA = g.xyz + 3 * A.atom, *RB = g.xyz + 3 * B.atom, *RC = g.xyz + 3 * C.atom,
               *RD = g.xyz + 3 * Dd.atom;
  quartet_bra_grad<LA, LB, LC, LD>(RA, RB, RC, RD, g.exps + A.off, g.coefs + A.off, A.np, g.exps + B.off,
                                   g.coefs + B.off, B.np, g.exps + C.off, g.coefs + C.off, C.np, g.exps + Dd.off,
                                   g.coefs + Dd.off, Dd.np, Gam, g.tab, wgt, gA, gB);
  quartet_bra_grad<LC, LD, LA, LB>(RC, RD, RA, RB, g.exps + C.off, g.coefs + C.off, C.np, g.exps + Dd.off,
                                   g.coefs + Dd.off, Dd.np, g.exps + A.off, g.coefs + A.off, A.np, g.exps + B.off,
                                   g.coefs + B.off, B.np, GamT, g.tab, wgt, gC, gD);
  // orientation (AB|CD) gives the A and B derivatives, (CD|AB) the C and D ones
  for (int x = 0; x < 3; ++x) {
    atomicAdd(&g.grad[3 * A.atom + x], gA[x]);
    atomicAdd(&g.grad[3 * B.atom + x], gB[x]);
    atomicAdd(&g.grad[3 * C.atom + x], gC[x]);
    atomicAdd(&g.grad[3 * Dd.atom + x], gD[x]);
  }
}

__global__ void __launch_bounds__(128) k_grad_2e(GradArgs g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nq) return;
  const int4 q = g.quartets[t];
  const double w = g.qweight[t];
  const int key = g.sh[q.x].L * 1000 + g.sh[q.y].L * 100 + g.sh[q.z].L * 10 + g.sh[q.w].L;
  switch (key) {
    case 0: quartet_grad<0, 0, 0, 0>(g, q, w); break;
    case 1000: quartet_grad<1, 0, 0, 0>(g, q, w); break;
    case 1010: quartet_grad<1, 0, 1, 0>(g, q, w); break;
    case 1100: quartet_grad<1, 1, 0, 0>(g, q, w); break;
    case 1110: quartet_grad<1, 1, 1, 0>(g, q, w); break;
    case 1111: quartet_grad<1, 1, 1, 1>(g, q, w); break;
    default: break;
  }
}

// ---------------------------------------------------------- one-electron ----
// Thread per function pair (a <= b): D-weighted derivatives of T and V (with
// the operator-centre term) and W-weighted derivatives of S.
__global__ void k_grad_1e(int nbf, int natoms, const double* __restrict__ xyz, const double* __restrict__ Z,
                          const int* __restrict__ fn, const double* __restrict__ coef, const double* __restrict__ expo,
                          const double* __restrict__ tab, const double* __restrict__ D, const double* __restrict__ W,
                          double* __restrict__ grad) {
  const int i = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nbf || j < i) return;
  const DevFn f = load_fn(fn, i), gfn = load_fn(fn, j);
  const double *A = xyz + 3 * f.atom, *B = xyz + 3 * gfn.atom;
  const double mult = (i == j) ? 1.0 : 2.0;
  const double dab = mult * D[(long)i * nbf + j], wab = mult * W[(long)i * nbf + j];
  const int L = f.l[0] + f.l[1] + f.l[2] + gfn.l[0] + gfn.l[1] + gfn.l[2] + 1;
  double gA[3] = {0, 0, 0};                    // d/dA of (D T - W S); d/dB = -d/dA
  double F[MD_LMAX + 2];
  double R[MD_D * MD_D * MD_D];
  for (int p1 = 0; p1 < f.np; ++p1)
    for (int p2 = 0; p2 < gfn.np; ++p2) {
      const double c1 = coef[f.off + p1], a = expo[f.off + p1];
      const double c2 = coef[gfn.off + p2], b = expo[gfn.off + p2];
      const double p = a + b, mu = a * b / p;
      const double cte = sqrt(GBHF_PI / p);
      double P[3], s[3][3][5];
      for (int x = 0; x < 3; ++x) {
        P[x] = (a * A[x] + b * B[x]) / p;
        const double ab = A[x] - B[x];
        // table up to i+1 on A and j+2 on B (kinetic)
        const double s00 = exp(-mu * ab * ab) * cte;
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
      auto T1 = [&](int x, int m, int nn) {   // kinetic 1-D term as in tab
        if (m < 0) return 0.0;
        return -2.0 * b * b * S1(x, m, nn + 2) + b * (2 * nn + 1) * S1(x, m, nn) -
               (nn >= 2 ? 0.5 * nn * (nn - 1) * S1(x, m, nn - 2) : 0.0);
      };
      for (int dir = 0; dir < 3; ++dir) {
        // d/dA_dir of S and T: replace axis dir factor by 2a f(i+1) - i f(i-1)
        double dS = c1 * c2, dT = 0;
        double sx[3], tx[3], dsx[3], dtx[3];
        for (int x = 0; x < 3; ++x) {
          const int li = f.l[x], lj = gfn.l[x];
          sx[x] = S1(x, li, lj);
          tx[x] = T1(x, li, lj);
          dsx[x] = 2 * a * S1(x, li + 1, lj) - li * S1(x, li - 1, lj);
          dtx[x] = 2 * a * T1(x, li + 1, lj) - li * T1(x, li - 1, lj);
        }
        dS = 1.0;
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
      // nuclear attraction: d/dA and d/dB of V^C, operator centre -(dA + dB)
      EAx E[3];
      for (int x = 0; x < 3; ++x) {
        const double ab = A[x] - B[x];
        e_axis(E[x], f.l[x] + 1 <= 2 ? f.l[x] + 1 : 2, gfn.l[x] + 1 <= 2 ? gfn.l[x] + 1 : 2, p, P[x] - A[x],
               P[x] - B[x], exp(-mu * ab * ab));
      }
      for (int cn = 0; cn < natoms; ++cn) {
        const double* Cc = xyz + 3 * cn;
        const double PC[3] = {P[0] - Cc[0], P[1] - Cc[1], P[2] - Cc[2]};
        boys_generic(false, nullptr, tab, L, p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]), F);
        hermite_r<MD_LMAX>(L, p, PC[0], PC[1], PC[2], F, R);
        const double vpref = -Z[cn] * c1 * c2 * 2.0 * (GBHF_PI / p) * dab;
        double dA[3] = {0, 0, 0}, dB[3] = {0, 0, 0};
        for (int dir = 0; dir < 3; ++dir) {
          int hi[3];
          for (int x = 0; x < 3; ++x) hi[x] = f.l[x] + gfn.l[x] + (x == dir ? 1 : 0);
          for (int t = 0; t <= hi[0]; ++t)
            for (int u = 0; u <= hi[1]; ++u)
              for (int v = 0; v <= hi[2]; ++v) {
                const int tt[3] = {t, u, v};
                double eA = 1, eB = 1;
                for (int x = 0; x < 3; ++x) {
                  const int li = f.l[x], lj = gfn.l[x];
                  if (x == dir) {
                    eA *= 2 * a * E[x].get(li + 1, lj, tt[x]) - li * E[x].get(li - 1, lj, tt[x]);
                    eB *= 2 * b * E[x].get(li, lj + 1, tt[x]) - lj * E[x].get(li, lj - 1, tt[x]);
                  } else {
                    const double e = E[x].get(li, lj, tt[x]);
                    eA *= e;
                    eB *= e;
                  }
                }
                const double r = R[(t * MD_D + u) * MD_D + v];
                dA[dir] += eA * r;
                dB[dir] += eB * r;
              }
        }
        for (int x = 0; x < 3; ++x) {
          atomicAdd(&grad[3 * f.atom + x], vpref * dA[x]);
          atomicAdd(&grad[3 * gfn.atom + x], vpref * dB[x]);
          atomicAdd(&grad[3 * cn + x], -vpref * (dA[x] + dB[x]));
        }
      }
    }
  for (int x = 0; x < 3; ++x) {
    atomicAdd(&grad[3 * f.atom + x], gA[x]);
    atomicAdd(&grad[3 * gfn.atom + x], -gA[x]);
  }
}

}  // namespace gbhf

using namespace gbhf;

// Host driver: D and W square (device), gradient into d_grad (3*natoms, device).
namespace gbhf {
gbhf_status gradient_dev(gbhf_ctx* c, const double* d_D, const double* d_W, double schwarz, double* d_grad) {
  const Basis& b = c->basis;
  if (!b.shells_ok || b.maxL > 1)
    return fail(c, GBHF_ERR_UNSUPPORTED, "gradient kernels need complete s/p shells");
  GBHF_TRY(ensure_boys_tables(c));
  GBHF_TRY(ensure_pairs(c));
  const int n = b.nbf, na = b.natoms;
  GBHF_CUDA(c, cudaMemsetAsync(d_grad, 0, 3 * na * sizeof(double), c->stream));
  // one-electron terms
  k_grad_1e<<<dim3((n + 63) / 64, n), 64, 0, c->stream>>>(n, na, c->d_xyz.p, c->d_Z.p, c->d_fn.p, c->d_coef.p,
                                                          c->d_exp.p, c->boys64.p, d_D, d_W, d_grad);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  // two-electron terms: unique shell quartets passing Schwarz
  const PairData& P = c->pairs;
  std::vector<int4> quart;
  std::vector<double> wq;
  for (int X = 0; X < NPCLS; ++X)
    for (int i = P.cls_start[X]; i < P.cls_start[X + 1]; ++i)
      for (int Y = 0; Y <= X; ++Y)
        for (int j = P.cls_start[Y]; j < P.cls_start[Y + 1]; ++j) {
          if (X == Y && j > i) break;
          if (P.hQ[i] * P.hQ[j] < schwarz) continue;
          const int A = P.hA[i], B = P.hB[i], C = P.hA[j], D = P.hB[j];
          quart.push_back(make_int4(A, B, C, D));
          wq.push_back((A == B ? 0.5 : 1.0) * (C == D ? 0.5 : 1.0) * (i == j ? 0.5 : 1.0));
        }
  const int nq = (int)quart.size();
  std::vector<GradShell> sh(b.shells.size());
  std::vector<double> ex, co;
  for (size_t s = 0; s < b.shells.size(); ++s) {
    sh[s].atom = b.shells[s].atom;
    sh[s].L = b.shells[s].L;
    sh[s].np = b.shells[s].np;
    sh[s].f0 = b.shells[s].f0;
    sh[s].off = (int)ex.size();
    ex.insert(ex.end(), b.shells[s].expo.begin(), b.shells[s].expo.end());
    co.insert(co.end(), b.shells[s].coef.begin(), b.shells[s].coef.end());
  }
  DBuf<int4> dq;
  DBuf<double> dw, dex, dco;
  DBuf<GradShell> dsh;
  GBHF_CUDA(c, dq.alloc(std::max(nq, 1)));
  GBHF_CUDA(c, dw.alloc(std::max(nq, 1)));
  GBHF_CUDA(c, dex.alloc(ex.size()));
  GBHF_CUDA(c, dco.alloc(co.size()));
  GBHF_CUDA(c, dsh.alloc(sh.size()));
  GBHF_CUDA(c, cudaMemcpyAsync(dq.p, quart.data(), nq * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dw.p, wq.data(), nq * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dex.p, ex.data(), ex.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dco.p, co.data(), co.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dsh.p, sh.data(), sh.size() * sizeof(GradShell), cudaMemcpyHostToDevice, c->stream));
  GradArgs g;
  g.nq = nq;
  g.quartets = dq.p;
  g.qweight = dw.p;
  g.sh = dsh.p;
  g.exps = dex.p;
  g.coefs = dco.p;
  g.xyz = c->d_xyz.p;
  g.D = d_D;
  g.n = n;
  g.tab = c->boys64.p;
  g.grad = d_grad;
  if (nq > 0) {
    k_grad_2e<<<(nq + 127) / 128, 128, 0, c->stream>>>(g);
    count_launch(c);
    GBHF_CUDA(c, cudaGetLastError());
  }
  // nuclear repulsion: d/dR_K sum_{K<L} Z_K Z_L / R_KL
  std::vector<double> gn(3 * na, 0.0);
  for (int k = 0; k < na; ++k)
    for (int l = 0; l < na; ++l) {
      if (l == k) continue;
      double d[3], r2 = 0;
      for (int x = 0; x < 3; ++x) {
        d[x] = b.xyz[3 * k + x] - b.xyz[3 * l + x];
        r2 += d[x] * d[x];
      }
      const double r3 = r2 * std::sqrt(r2);
      for (int x = 0; x < 3; ++x) gn[3 * k + x] -= b.Z[k] * b.Z[l] * d[x] / r3;
    }
  DBuf<double> dgn;
  GBHF_CUDA(c, dgn.alloc(3 * na));
  GBHF_CUDA(c, cudaMemcpyAsync(dgn.p, gn.data(), 3 * na * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(axpby(c, 3 * (size_t)na, 1.0, d_grad, 1.0, dgn.p, d_grad));
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
