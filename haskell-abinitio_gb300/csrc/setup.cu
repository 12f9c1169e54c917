// Basis upload, Boys tables and shell-pair data for the direct J/K build.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>

#include "gbhf_internal.h"

namespace gbhf {

thread_local DevPool* tls_pool = nullptr;

gbhf_status fail(gbhf_ctx* c, gbhf_status s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}

gbhf_status cuda_fail(gbhf_ctx* c, cudaError_t e, const char* where) {
  std::string m = std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ") in " + where;
  return fail(c, GBHF_ERR_CUDA, m);
}

static int ncart(int L) { return (L + 1) * (L + 2) / 2; }

// Group CGFs into shells: consecutive CGFs on one atom with the same total
// angular momentum and identical exponents, in the Cartesian order x, y, z and
// xx, xy, xz, yy, yz, zz (the order createCGF emits, BasisSet/FetchBasis.hs:50-59).
// The components of a d shell differ in their primitive normalisation
// (normCoeff, BasisSet/NormalizeBasis.hs:37-59: a factor 1/sqrt(prod (2l_k-1)!!)),
// so their coefficients need only be proportional: the shell keeps the first
// component's coefficients and the ratio of every component as its scale.
static void group_shells(Basis& b) {
  b.shells.clear();
  b.shells_ok = true;
  b.maxL = 0;
  const int n = b.nbf;
  int i = 0;
  static const int cart[10][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0},
                                  {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}};
  while (i < n) {
    const int* l = &b.cgf_lxyz[3 * i];
    const int L = l[0] + l[1] + l[2];
    b.maxL = std::max(b.maxL, L);
    Shell s;
    s.atom = b.cgf_atom[i];
    s.L = L;
    s.np = b.cgf_nprim[i];
    s.ncomp = ncart(L);
    s.f0 = i;
    s.expo.assign(b.prim_exp.begin() + b.cgf_off[i], b.prim_exp.begin() + b.cgf_off[i] + s.np);
    s.coef.assign(b.prim_coef.begin() + b.cgf_off[i], b.prim_coef.begin() + b.cgf_off[i] + s.np);
    bool ok = L <= 2;
    int take = ok ? s.ncomp : 1;
    if (i + take > n) ok = false;
    const int c0 = L == 0 ? 0 : (L == 1 ? 1 : 4);   // first row of this L in cart
    for (int c = 0; ok && c < take; ++c) {
      const int j = i + c;
      const int* lj = &b.cgf_lxyz[3 * j];
      if (b.cgf_atom[j] != s.atom || b.cgf_nprim[j] != s.np) ok = false;
      if (ok && !(lj[0] == cart[c0 + c][0] && lj[1] == cart[c0 + c][1] && lj[2] == cart[c0 + c][2])) ok = false;
      const double r = (ok && s.coef[0] != 0.0) ? b.prim_coef[b.cgf_off[j]] / s.coef[0] : 1.0;
      for (int k = 0; ok && k < s.np; ++k) {
        const double cj = b.prim_coef[b.cgf_off[j] + k];
        if (b.prim_exp[b.cgf_off[j] + k] != s.expo[k]) ok = false;
        if (L <= 1 ? cj != s.coef[k] : std::fabs(cj - r * s.coef[k]) > 1e-13 * std::fabs(cj)) ok = false;
      }
      if (ok) s.scale[c] = r;
    }
    if (!ok) {
      if (b.shells_ok) {
        b.shell_msg = "basis function " + std::to_string(i) +
                      " does not start a complete s, p or d shell (Cartesian components in order, shared"
                      " exponents, proportional coefficients)";
      }
      b.shells_ok = false;
      s.ncomp = 1;
      take = 1;
    }
    b.shells.push_back(std::move(s));
    i += take;
  }
}

gbhf_status build_basis(gbhf_ctx* c, int n_atoms, const double* xyz, const double* Z, int n_cgf, const int* cgf_atom,
                        const int* cgf_lxyz, const int* cgf_nprim, const double* coef, const double* expo) {
  const int aoff[2] = {0, n_atoms}, foff[2] = {0, n_cgf};
  return build_basis_mols(c, n_atoms, xyz, Z, n_cgf, cgf_atom, cgf_lxyz, cgf_nprim, coef, expo, 1, aoff, foff);
}

gbhf_status build_basis_mols(gbhf_ctx* c, int n_atoms, const double* xyz, const double* Z, int n_cgf,
                             const int* cgf_atom, const int* cgf_lxyz, const int* cgf_nprim, const double* coef,
                             const double* expo, int nmol, const int* atom_off, const int* cgf_off) {
  if (n_atoms <= 0 || n_cgf <= 0 || !xyz || !Z || !cgf_atom || !cgf_lxyz || !cgf_nprim || !coef || !expo)
    return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_set_basis: empty basis or null pointer");
  if (nmol < 1 || !atom_off || !cgf_off || atom_off[0] != 0 || cgf_off[0] != 0 || atom_off[nmol] != n_atoms ||
      cgf_off[nmol] != n_cgf)
    return fail(c, GBHF_ERR_BAD_INPUT, "molecule partition does not cover the atoms and functions");
  Basis b;
  b.natoms = n_atoms;
  b.nbf = n_cgf;
  b.nmol = nmol;
  b.mol_atom_off.assign(atom_off, atom_off + nmol + 1);
  b.mol_fn_off.assign(cgf_off, cgf_off + nmol + 1);
  b.mol_moff.resize(nmol + 1);
  b.mol_moff[0] = 0;
  for (int m = 0; m < nmol; ++m) {
    const int a0 = atom_off[m], a1 = atom_off[m + 1], f0 = cgf_off[m], f1 = cgf_off[m + 1];
    if (a1 <= a0 || f1 <= f0)
      return fail(c, GBHF_ERR_BAD_INPUT, "molecule " + std::to_string(m) + " has no atoms or no functions");
    for (int i = f0; i < f1; ++i)
      if (cgf_atom[i] < a0 || cgf_atom[i] >= a1)
        return fail(c, GBHF_ERR_BAD_INPUT, "a CGF of molecule " + std::to_string(m) + " sits on another molecule's atom");
    b.mol_moff[m + 1] = b.mol_moff[m] + (long long)(f1 - f0) * (f1 - f0);
  }
  b.stacked = b.mol_moff[nmol];
  b.xyz.assign(xyz, xyz + 3 * n_atoms);
  b.Z.assign(Z, Z + n_atoms);
  b.cgf_atom.assign(cgf_atom, cgf_atom + n_cgf);
  b.cgf_lxyz.assign(cgf_lxyz, cgf_lxyz + 3 * n_cgf);
  b.cgf_nprim.assign(cgf_nprim, cgf_nprim + n_cgf);
  b.cgf_off.resize(n_cgf + 1);
  b.cgf_off[0] = 0;
  for (int i = 0; i < n_cgf; ++i) {
    if (cgf_atom[i] < 0 || cgf_atom[i] >= n_atoms)
      return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_set_basis: CGF atom index out of range");
    if (cgf_nprim[i] <= 0 || cgf_nprim[i] > 6)
      return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_set_basis: 1..6 primitives per CGF supported");
    for (int x = 0; x < 3; ++x)
      if (cgf_lxyz[3 * i + x] < 0 || cgf_lxyz[3 * i + x] > 2)
        return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_set_basis: Cartesian exponent out of range (s, p, d only)");
    if (cgf_lxyz[3 * i] + cgf_lxyz[3 * i + 1] + cgf_lxyz[3 * i + 2] > 2)
      return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_set_basis: angular momentum above d");
    b.cgf_off[i + 1] = b.cgf_off[i] + cgf_nprim[i];
  }
  const int nprim = b.cgf_off[n_cgf];
  b.prim_coef.assign(coef, coef + nprim);
  b.prim_exp.assign(expo, expo + nprim);
  for (int k = 0; k < nprim; ++k)
    if (!(expo[k] > 0) || !std::isfinite(coef[k]))
      return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_set_basis: exponents must be positive and coefficients finite");
  for (int k = 0; k < 3 * n_atoms; ++k)
    if (!std::isfinite(xyz[k])) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_set_basis: non-finite coordinate");
  group_shells(b);
  for (auto& sh : b.shells) {
    int m = 0;
    while (m + 1 < nmol && sh.f0 >= cgf_off[m + 1]) ++m;
    sh.mol = m;
  }
  c->basis = std::move(b);
  const Basis& B = c->basis;
  // device copies (function level)
  std::vector<int> fn(6 * n_cgf);
  for (int i = 0; i < n_cgf; ++i) {
    fn[6 * i] = B.cgf_atom[i];
    fn[6 * i + 1] = B.cgf_lxyz[3 * i];
    fn[6 * i + 2] = B.cgf_lxyz[3 * i + 1];
    fn[6 * i + 3] = B.cgf_lxyz[3 * i + 2];
    fn[6 * i + 4] = B.cgf_nprim[i];
    fn[6 * i + 5] = B.cgf_off[i];
  }
  GBHF_CUDA(c, c->d_xyz.alloc(3 * n_atoms));
  GBHF_CUDA(c, c->d_Z.alloc(n_atoms));
  GBHF_CUDA(c, c->d_fn.alloc(6 * n_cgf));
  GBHF_CUDA(c, c->d_coef.alloc(nprim));
  GBHF_CUDA(c, c->d_exp.alloc(nprim));
  GBHF_CUDA(c, cudaMemcpyAsync(c->d_xyz.p, B.xyz.data(), 3 * n_atoms * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->d_Z.p, B.Z.data(), n_atoms * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->d_fn.p, fn.data(), 6 * n_cgf * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->d_coef.p, B.prim_coef.data(), nprim * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->d_exp.p, B.prim_exp.data(), nprim * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->basis_dev = true;
  c->pairs_ready = false;
  c->basis_gen += 1;
  c->tasks.thr_all = -1;
  c->tasks.thr64 = -1;
  return GBHF_OK;
}

// Exact Boys function F_0 .. F_(BOYS_NCOL-1)(x) in extended precision: the power series
//   F_m(x) = exp(-x) sum_k (2x)^k / ((2m+1)(2m+3)...(2m+2k+1))
// (all terms positive, so no cancellation) for the highest order, terms until
// below 1e-22 of the sum, then the downward
// recursion F_m = (2x F_(m+1) + exp(-x)) / (2m + 1), which is stable.  One
// series per node (long double is software-emulated quad precision on some
// hosts, so the tables cost one series per node rather than one per order).
static void boys_row_host(double xd, double* out) {
  const long double x = xd;
  const int mt = BOYS_NCOL - 1;
  long double term = 1.0L / (2 * mt + 1), sum = term;
  for (int k = 1; k < 4000; ++k) {
    term *= 2 * x / (2 * mt + 2 * k + 1);
    sum += term;
    if (term < sum * 1e-22L) break;
  }
  const long double ex = expl(-x);
  long double f = ex * sum;
  out[mt] = (double)f;
  for (int m = mt - 1; m >= 0; --m) {
    f = (2 * x * f + ex) / (2 * m + 1);
    out[m] = (double)f;
  }
}

// The host tables, computed once per process (the series run in long double,
// software quad precision on some hosts) and uploaded to every context.
struct BoysHostTables {
  std::vector<double> t64, h64;
  std::vector<float> t32, h32;
};

static BoysHostTables build_boys_host_tables() {
  BoysHostTables bt;
  std::vector<double>& t64 = bt.t64;
  t64.resize((size_t)BOYS64_NROW * BOYS_NCOL);
  std::vector<float>& t32 = bt.t32;
  t32.resize((size_t)BOYS32_NROW * BOYS_NCOL);
  std::vector<double> t32d((size_t)BOYS32_NROW * BOYS_NCOL);   // the FP32 nodes' values before rounding
  for (int j = 0; j < BOYS64_NROW; ++j) boys_row_host(j * BOYS64_H, t64.data() + (size_t)j * BOYS_NCOL);
  for (int j = 0; j < BOYS32_NROW; ++j) {
    const float tj = (float)j * BOYS32_H;   // the node the device forms in float
    boys_row_host((double)tj, t32d.data() + (size_t)j * BOYS_NCOL);
    for (int m = 0; m < BOYS_NCOL; ++m) t32[(size_t)j * BOYS_NCOL + m] = (float)t32d[(size_t)j * BOYS_NCOL + m];
  }
  // Horner tables per order L: row j = [F_(L+k)(T_j)/k!, k < NT][exp(-T_j)/k!, k < NT]
  std::vector<double>& h64 = bt.h64;
  h64.assign((size_t)(BOYSH_LMAX + 1) * BOYS64_NROW * BOYSH64_STRIDE, 0.0);
  std::vector<float>& h32 = bt.h32;
  h32.assign((size_t)(BOYSH_LMAX + 1) * BOYS32_NROW * BOYSH32_STRIDE, 0.0f);
  for (int L = 0; L <= BOYSH_LMAX; ++L) {
    for (int j = 0; j < BOYS64_NROW; ++j) {
      double* row = h64.data() + ((size_t)L * BOYS64_NROW + j) * BOYSH64_STRIDE;
      double inv_fact = 1.0;
      for (int k = 0; k < BOYS64_NTERM; ++k) {
        if (k > 0) inv_fact /= k;
        row[k] = t64[(size_t)j * BOYS_NCOL + L + k] * inv_fact;
        row[BOYS64_NTERM + k] = std::exp(-j * BOYS64_H) * inv_fact;
      }
      row[2 * BOYS64_NTERM] = j * BOYS64_H;   // the node itself
    }
    for (int j = 0; j < BOYS32_NROW; ++j) {
      float* row = h32.data() + ((size_t)L * BOYS32_NROW + j) * BOYSH32_STRIDE;
      const double tj = (double)((float)j * BOYS32_H);   // the node the device forms in float
      double inv_fact = 1.0;
      for (int k = 0; k < BOYS32_NTERM; ++k) {
        if (k > 0) inv_fact /= k;
        row[k] = (float)(t32d[(size_t)j * BOYS_NCOL + L + k] * inv_fact);
        row[BOYS32_NTERM + k] = (float)(std::exp(-tj) * inv_fact);
      }
    }
  }
  return bt;
}

static const BoysHostTables& boys_host_tables() {
  static const BoysHostTables bt = build_boys_host_tables();   // thread-safe one-time initialisation
  return bt;
}

gbhf_status ensure_boys_tables(gbhf_ctx* c) {
  if (c->boys64.p && c->boys32.p && c->boysh64.p && c->boysh32.p) return GBHF_OK;
  const BoysHostTables& bt = boys_host_tables();
  const std::vector<double>& t64 = bt.t64;
  const std::vector<float>& t32 = bt.t32;
  const std::vector<double>& h64 = bt.h64;
  const std::vector<float>& h32 = bt.h32;
  GBHF_CUDA(c, c->boys64.alloc(t64.size()));
  GBHF_CUDA(c, c->boys32.alloc(t32.size()));
  GBHF_CUDA(c, c->boysh64.alloc(h64.size()));
  GBHF_CUDA(c, c->boysh32.alloc(h32.size()));
  GBHF_CUDA(c, cudaMemcpyAsync(c->boys64.p, t64.data(), t64.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->boys32.p, t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->boysh64.p, h64.data(), h64.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->boysh32.p, h32.data(), h32.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

static int pair_class(int la, int lb) { return pair_class_of(la, lb); }

// Fields of primitive pair k = ia*np_B + ib of shells (A, B).
// K' = sqrt(2 pi^(5/2)) c_a c_b exp(-mu |AB|^2) / p, so the product of a bra
// and a ket K' times 1/sqrt(p+q) is the whole ERI prefactor.  sh: per shell
// (atom, primitives, offset of its first CGF's primitives in coef/expo).
__device__ __forceinline__ void pair_prim_fields(const int4* __restrict__ sh, const double* __restrict__ xyz,
                                                 const double* __restrict__ coef, const double* __restrict__ expo,
                                                 int A, int B, int k, double* f) {
  const int4 sa = sh[A], sb = sh[B];
  const int ia = k / sb.y, ib = k - ia * sb.y;
  const double* RA = xyz + 3 * sa.x;
  const double* RB = xyz + 3 * sb.x;
  double r2 = 0;
  for (int x = 0; x < 3; ++x) r2 += (RA[x] - RB[x]) * (RA[x] - RB[x]);
  const double ea = expo[sa.z + ia], eb = expo[sb.z + ib];
  const double p = ea + eb, mu = ea * eb / p;
  f[BRA_P] = p;
  f[BRA_INVP] = 1.0 / p;
  for (int x = 0; x < 3; ++x) {
    const double Px = (ea * RA[x] + eb * RB[x]) / p;
    f[BRA_PX + x] = Px;
    f[BRA_PAX + x] = Px - RA[x];
    f[BRA_PBX + x] = Px - RB[x];
  }
  f[BRA_K] = sqrt(TWO_PI_2P5) * coef[sa.z + ia] * coef[sb.z + ib] * exp(-mu * r2) / p;
  f[BRA_AEXP] = ea;
}

// Pair-contiguous FP64 fields of pairs (pA, pB) at poff (the Schwarz pass).
__global__ void k_pair_fields(int np, const int* __restrict__ pA, const int* __restrict__ pB,
                              const int* __restrict__ poff, const int4* __restrict__ sh,
                              const double* __restrict__ xyz, const double* __restrict__ coef,
                              const double* __restrict__ expo, long long npp, double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const int A = pA[t], B = pB[t];
  const int K = sh[A].y * sh[B].y;
  double f[BRA_NFIELD];
  for (int k = 0; k < K; ++k) {
    pair_prim_fields(sh, xyz, coef, expo, A, B, k, f);
    for (int fl = 0; fl < BRA_NFIELD; ++fl) out[(long long)fl * npp + poff[t] + k] = f[fl];
  }
}

// Final layouts of the sorted pairs: bra (pair-contiguous) and ket
// (segment-transposed: primitive k of pair t at data_off + k*len + (t - start)),
// FP64 and FP32.
__global__ void k_pair_layouts(int np, const int* __restrict__ pA, const int* __restrict__ pB,
                               const int* __restrict__ poff, const int* __restrict__ kseg,
                               const int4* __restrict__ seg, const int4* __restrict__ sh,
                               const double* __restrict__ xyz, const double* __restrict__ coef,
                               const double* __restrict__ expo, long long npp, double* __restrict__ bra64,
                               double* __restrict__ ket64, float* __restrict__ bra32, float* __restrict__ ket32) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const int A = pA[t], B = pB[t];
  const int K = sh[A].y * sh[B].y;
  const int4 sg = seg[kseg[t]];
  const long long len = sg.y - sg.x;
  double f[BRA_NFIELD];
  for (int k = 0; k < K; ++k) {
    pair_prim_fields(sh, xyz, coef, expo, A, B, k, f);
    const long long bi = (long long)poff[t] + k, ki = (long long)sg.w + k * len + (t - sg.x);
    for (int fl = 0; fl < BRA_NFIELD; ++fl) {
      bra64[(long long)fl * npp + bi] = f[fl];
      ket64[(long long)fl * npp + ki] = f[fl];
      bra32[(long long)fl * npp + bi] = (float)f[fl];
      ket32[(long long)fl * npp + ki] = (float)f[fl];
    }
  }
}

gbhf_status ensure_pairs(gbhf_ctx* c) {
  if (c->pairs_ready) return GBHF_OK;
  const auto t_pairs = std::chrono::steady_clock::now();
  const Basis& b = c->basis;
  if (!c->basis_dev) return fail(c, GBHF_ERR_BAD_INPUT, "no basis set");
  if (!b.shells_ok || b.maxL > 2)
    return fail(c, GBHF_ERR_UNSUPPORTED,
                "direct J/K kernels need complete s, p and d shells: " +
                    (b.shell_msg.empty() ? std::string("functions above d present") : b.shell_msg));
  GBHF_TRY(ensure_boys_tables(c));
  GBHF_TRY(ensure_shell_arrays(c));   // component scales for the d-class Schwarz bounds
  const int ns = (int)b.shells.size();
  // shell table for the device: atom, primitives, first primitive of the shell's first CGF
  std::vector<int4> shv(ns);
  for (int s2 = 0; s2 < ns; ++s2) {
    const Shell& sh = b.shells[s2];
    shv[s2] = make_int4(sh.atom, sh.np, b.cgf_off[sh.f0], 0);
  }
  DBuf<int4> dsh;
  GBHF_CUDA(c, dsh.alloc(std::max(ns, 1)));
  GBHF_CUDA(c, cudaMemcpyAsync(dsh.p, shv.data(), ns * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
  // 1. all pairs (la > lb, or la == lb and A >= B) of shells of one molecule,
  //    grouped by class as they are generated (counting sort)
  std::vector<int> A, B, cls;
  for (int s0 = 0; s0 < ns;) {
    int s1 = s0;
    while (s1 < ns && b.shells[s1].mol == b.shells[s0].mol) ++s1;
    for (int a = s0; a < s1; ++a)
      for (int bb = s0; bb < s1; ++bb) {
        const int la = b.shells[a].L, lb = b.shells[bb].L;
        if (la > lb || (la == lb && a >= bb)) {
          A.push_back(a);
          B.push_back(bb);
          cls.push_back(pair_class(la, lb));
        }
      }
    s0 = s1;
  }
  const int np = (int)A.size();
  std::vector<int> ord0(np);
  int cs0[NPCLS + 1] = {};
  {
    std::vector<int> cnt(NPCLS + 1, 0);
    for (int t = 0; t < np; ++t) ++cnt[cls[t] + 1];
    for (int cl = 0; cl < NPCLS; ++cl) cnt[cl + 1] += cnt[cl];
    for (int cl = 0; cl <= NPCLS; ++cl) cs0[cl] = cnt[cl];
    for (int t = 0; t < np; ++t) ord0[cnt[cls[t]]++] = t;
  }
  // 2. Schwarz bounds on the device, pairs grouped by class (class code, FP64)
  std::vector<double> Q(np);
  {
    std::vector<int> A0(np), B0(np), K0(np), off0(np);
    size_t npp0 = 0;
    for (int t = 0; t < np; ++t) {
      A0[t] = A[ord0[t]];
      B0[t] = B[ord0[t]];
      K0[t] = b.shells[A0[t]].np * b.shells[B0[t]].np;
      off0[t] = (int)npp0;
      npp0 += K0[t];
    }
    DBuf<int> dK, doff, dA0, dB0;
    DBuf<double> dQ, dbra;
    GBHF_CUDA(c, dK.alloc(std::max(np, 1)));
    GBHF_CUDA(c, doff.alloc(std::max(np, 1)));
    GBHF_CUDA(c, dA0.alloc(std::max(np, 1)));
    GBHF_CUDA(c, dB0.alloc(std::max(np, 1)));
    GBHF_CUDA(c, dQ.alloc(std::max(np, 1)));
    GBHF_CUDA(c, dbra.alloc(std::max<size_t>((size_t)BRA_NFIELD * npp0, 1)));
    GBHF_CUDA(c, cudaMemcpyAsync(dK.p, K0.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(doff.p, off0.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(dA0.p, A0.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(dB0.p, B0.data(), np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    if (np > 0) {
      k_pair_fields<<<(np + 127) / 128, 128, 0, c->stream>>>(np, dA0.p, dB0.p, doff.p, dsh.p, c->d_xyz.p,
                                                             c->d_coef.p, c->d_exp.p, (long long)npp0, dbra.p);
      count_launch(c);
      GBHF_CUDA(c, cudaGetLastError());
    }
    GBHF_TRY(schwarz_classes_dev(c, cs0, dK.p, doff.p, dbra.p, (long long)npp0, dQ.p));
    GBHF_TRY(schwarz_dclasses_dev(c, cs0, dA0.p, dB0.p, dK.p, doff.p, dbra.p, (long long)npp0, dQ.p));
    std::vector<double> Q0(np);
    GBHF_CUDA(c, cudaMemcpyAsync(Q0.data(), dQ.p, np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int t = 0; t < np; ++t) Q[ord0[t]] = Q0[t];
  }
  // 3. order: class, molecule, primitive-pair count descending, Q descending
  std::vector<int> order(np), Kp(np), molp(np);
  for (int t = 0; t < np; ++t) {
    Kp[t] = b.shells[A[t]].np * b.shells[B[t]].np;
    molp[t] = b.shells[A[t]].mol;
  }
  // ord0 holds the pairs grouped by class, each class in generation order, i.e.
  // by molecule when the shells come molecule by molecule: then only the runs of
  // one (class, molecule) need sorting
  auto within = [&](int x, int y) {
    if (Kp[x] != Kp[y]) return Kp[x] > Kp[y];
    if (Q[x] != Q[y]) return Q[x] > Q[y];
    return x < y;
  };
  bool mol_ordered = true;
  for (int s2 = 1; s2 < ns; ++s2) mol_ordered &= b.shells[s2].mol >= b.shells[s2 - 1].mol;
  if (mol_ordered) {
    // each run sorted as compact (K, Q, index) records: the comparisons stay in cache
    struct PairKey {
      int K;
      double Q;
      int idx;
    };
    std::vector<PairKey> keys;
    order = ord0;
    for (int r0 = 0; r0 < np;) {
      int r1 = r0 + 1;
      while (r1 < np && cls[order[r1]] == cls[order[r0]] && molp[order[r1]] == molp[order[r0]]) ++r1;
      keys.resize(r1 - r0);
      for (int t = r0; t < r1; ++t) keys[t - r0] = {Kp[order[t]], Q[order[t]], order[t]};
      std::sort(keys.begin(), keys.end(), [](const PairKey& x, const PairKey& y) {
        if (x.K != y.K) return x.K > y.K;
        if (x.Q != y.Q) return x.Q > y.Q;
        return x.idx < y.idx;
      });
      for (int t = r0; t < r1; ++t) order[t] = keys[t - r0].idx;
      r0 = r1;
    }
  } else {
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int x, int y) {
      if (cls[x] != cls[y]) return cls[x] < cls[y];
      if (molp[x] != molp[y]) return molp[x] < molp[y];
      return within(x, y);
    });
  }
  PairData& P = c->pairs;
  P.npairs = np;
  P.hA.resize(np);
  P.hB.resize(np);
  P.hK.resize(np);
  P.hQ.resize(np);
  P.hPoff.resize(np);
  P.hSeg.resize(np);
  for (int cl = 0; cl < NPCLS; ++cl) P.segs[cl].clear();
  for (int cl = 0; cl <= NPCLS; ++cl) P.cls_start[cl] = np;
  size_t poff = 0;
  for (int t = 0; t < np; ++t) {
    const int o = order[t];
    P.hA[t] = A[o];
    P.hB[t] = B[o];
    P.hK[t] = Kp[o];
    P.hQ[t] = Q[o];
    P.hPoff[t] = (int)poff;
    poff += P.hK[t];
    const int cl = cls[o];
    if (P.cls_start[cl] == np) P.cls_start[cl] = t;
    auto& sg = P.segs[cl];
    if (sg.empty() || sg.back().K != P.hK[t] || molp[order[sg.back().start]] != molp[o])
      sg.push_back({t, t + 1, P.hK[t], 0});
    else sg.back().end = t + 1;
  }
  for (int cl = NPCLS - 1; cl >= 0; --cl)
    if (P.cls_start[cl] == np && cl + 1 <= NPCLS) P.cls_start[cl] = P.cls_start[cl + 1];
  P.nprim_pairs = poff;
  // segment table (global) and ket-layout offsets
  std::vector<int4> seginfo;
  size_t koff = 0;
  for (int cl = 0; cl < NPCLS; ++cl) {
    P.seg_cls_start[cl] = (int)seginfo.size();
    for (auto& sgm : P.segs[cl]) {
      sgm.data_off = (int)koff;
      koff += (size_t)(sgm.end - sgm.start) * sgm.K;
      for (int t = sgm.start; t < sgm.end; ++t) P.hSeg[t] = (int)seginfo.size();
      seginfo.push_back(make_int4(sgm.start, sgm.end, sgm.K, sgm.data_off));
    }
  }
  P.seg_cls_start[NPCLS] = (int)seginfo.size();
  P.nseg_total = (int)seginfo.size();
  // segments of each (class, molecule); empty ranges for absent classes
  const int nmol = b.nmol;
  P.hmseg.assign(2 * (size_t)NPCLS * nmol, 0);
  for (int cl = 0; cl < NPCLS; ++cl)
    for (int m = 0; m < nmol; ++m) P.hmseg[2 * (cl * nmol + m)] = P.hmseg[2 * (cl * nmol + m) + 1] = P.seg_cls_start[cl];
  for (int cl = 0; cl < NPCLS; ++cl)
    for (int sidx = P.seg_cls_start[cl]; sidx < P.seg_cls_start[cl + 1]; ++sidx) {
      const int m = b.shells[P.hA[seginfo[sidx].x]].mol;
      int* r = &P.hmseg[2 * (cl * nmol + m)];
      if (r[1] == r[0]) r[0] = sidx;
      r[1] = sidx + 1;
    }
  std::vector<int> pmol(np);
  for (int t = 0; t < np; ++t) pmol[t] = b.shells[P.hA[t]].mol;
  // 4. primitive-pair data, built on the device in both layouts and precisions
  const size_t npp = poff;
  const size_t nf = std::max<size_t>((size_t)BRA_NFIELD * npp, 1);
  GBHF_CUDA(c, P.A.alloc(std::max(np, 1)));
  GBHF_CUDA(c, P.B.alloc(std::max(np, 1)));
  GBHF_CUDA(c, P.K.alloc(std::max(np, 1)));
  GBHF_CUDA(c, P.poff.alloc(std::max(np, 1)));
  GBHF_CUDA(c, P.kseg.alloc(std::max(np, 1)));
  GBHF_CUDA(c, P.Q.alloc(std::max(np, 1)));
  GBHF_CUDA(c, P.seg_info.alloc(std::max<size_t>(seginfo.size(), 1)));
  GBHF_CUDA(c, P.mol.alloc(std::max(np, 1)));
  GBHF_CUDA(c, P.mseg.alloc(std::max<size_t>(P.hmseg.size(), 1)));
  GBHF_CUDA(c, P.bra64.alloc(nf));
  GBHF_CUDA(c, P.ket64.alloc(nf));
  GBHF_CUDA(c, P.bra32.alloc(nf));
  GBHF_CUDA(c, P.ket32.alloc(nf));
  auto up = [&](void* d, const void* h, size_t bytes) {
    return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->stream);
  };
  GBHF_CUDA(c, up(P.A.p, P.hA.data(), np * sizeof(int)));
  GBHF_CUDA(c, up(P.B.p, P.hB.data(), np * sizeof(int)));
  GBHF_CUDA(c, up(P.K.p, P.hK.data(), np * sizeof(int)));
  GBHF_CUDA(c, up(P.poff.p, P.hPoff.data(), np * sizeof(int)));
  GBHF_CUDA(c, up(P.kseg.p, P.hSeg.data(), np * sizeof(int)));
  GBHF_CUDA(c, up(P.Q.p, P.hQ.data(), np * sizeof(double)));
  std::vector<float> qf(P.hQ.begin(), P.hQ.end());
  GBHF_CUDA(c, P.Qf.alloc(std::max(np, 1)));
  GBHF_CUDA(c, up(P.Qf.p, qf.data(), np * sizeof(float)));
  GBHF_CUDA(c, up(P.seg_info.p, seginfo.data(), seginfo.size() * sizeof(int4)));
  GBHF_CUDA(c, up(P.mol.p, pmol.data(), np * sizeof(int)));
  GBHF_CUDA(c, up(P.mseg.p, P.hmseg.data(), P.hmseg.size() * sizeof(int)));
  if (np > 0) {
    k_pair_layouts<<<(np + 127) / 128, 128, 0, c->stream>>>(np, P.A.p, P.B.p, P.poff.p, P.kseg.p, P.seg_info.p, dsh.p,
                                                            c->d_xyz.p, c->d_coef.p, c->d_exp.p, (long long)npp,
                                                            P.bra64.p, P.ket64.p, P.bra32.p, P.ket32.p);
    count_launch(c);
    GBHF_CUDA(c, cudaGetLastError());
  }
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->pairs_ready = true;
  c->prof.ph_pairs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_pairs).count();
  return GBHF_OK;
}

}  // namespace gbhf
