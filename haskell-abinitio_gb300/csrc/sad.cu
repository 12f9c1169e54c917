// Superposition-of-atomic-densities (SAD) initial density.
//
// The reference starts from the Harris functional or the core Hamiltonian
// (HartreeFock/HartreeFock.hs:128-149); for clusters of tens of molecules the
// core guess with DIIS from the first step often fails to converge.  SAD takes
// the block-diagonal density of free atoms instead: for every distinct atom
// (element and basis functions) a spherically averaged fractional-occupation
// RHF of the single atom is run once on the device (stored ERIs, Jacobi
// eigen-solve) and cached in the context; the molecular guess is the
// block-diagonal assembly of those atomic densities.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gbhf_internal.h"

namespace gbhf {

__global__ void k_sad_scale_cols(int n, const double* __restrict__ C, const double* __restrict__ occ,
                                 double* __restrict__ out) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  out[(long)i * n + j] = C[(long)i * n + j] * occ[j];
}

// Row i (global function) of its molecule's block of the stacked densities:
// D[i][j] = block of atom(i) at (loc(i), loc(j)) when atom(i) == atom(j), else 0.
__global__ void k_sad_assemble(const int* __restrict__ fmol, const int* __restrict__ mfo,
                               const long long* __restrict__ moff, const int* __restrict__ fatom,
                               const int* __restrict__ floc, const int* __restrict__ boff,
                               const int* __restrict__ bdim, const double* __restrict__ blocks,
                               double* __restrict__ D) {
  const int i = blockIdx.y;
  const int m = fmol[i], f0 = mfo[m], n = mfo[m + 1] - f0;
  const int jl = blockIdx.x * blockDim.x + threadIdx.x;
  if (jl >= n) return;
  const int j = f0 + jl, a = fatom[i];
  double v = 0.0;
  if (fatom[j] == a) v = blocks[boff[a] + floc[i] * bdim[a] + floc[j]];
  D[moff[m] + (long long)(i - f0) * n + jl] = v;
}

// Key of atom a: nuclear charge and its functions (Cartesian exponents,
// contraction coefficients and exponents) in basis order.
static std::string atom_key(const Basis& b, int a, std::vector<int>& fns) {
  fns.clear();
  std::string k;
  auto put = [&](const void* p, size_t s) { k.append(static_cast<const char*>(p), s); };
  put(&b.Z[a], sizeof(double));
  int m = 0;
  while (m + 1 < b.nmol && a >= b.mol_atom_off[m + 1]) ++m;
  for (int i = b.mol_fn_off[m]; i < b.mol_fn_off[m + 1]; ++i) {
    if (b.cgf_atom[i] != a) continue;
    fns.push_back(i);
    put(&b.cgf_lxyz[3 * i], 3 * sizeof(int));
    put(&b.cgf_nprim[i], sizeof(int));
    put(&b.prim_coef[b.cgf_off[i]], b.cgf_nprim[i] * sizeof(double));
    put(&b.prim_exp[b.cgf_off[i]], b.cgf_nprim[i] * sizeof(double));
  }
  return k;
}

// Aufbau occupations (2 electrons per orbital) for nel electrons, shared
// equally by orbitals whose energies agree to 1e-5 Eh (a partly filled
// degenerate shell, e.g. O 2p^4 -> 4/3 per p orbital, keeps the density
// spherical).
static void frac_occupations(const std::vector<double>& eps, double nel, std::vector<double>& occ) {
  const int n = (int)eps.size();
  occ.assign(n, 0.0);
  double left = nel;
  for (int i = 0; i < n && left > 1e-12;) {
    int j = i;
    while (j + 1 < n && std::fabs(eps[j + 1] - eps[i]) < 1e-5) ++j;
    const int g = j - i + 1;
    const double take = std::min(left, 2.0 * g);
    for (int k = i; k <= j; ++k) occ[k] = take / g;
    left -= take;
    i = j + 1;
  }
}

// Fractional-occupation RHF of one neutral atom at the origin (functions
// `fns` of the molecular basis), density in `block` (nf x nf, row-major).
static gbhf_status atomic_density(gbhf_ctx* c, gbhf_ctx* sub, const Basis& b, int a, const std::vector<int>& fns,
                                  std::vector<double>& block) {
  const int nf = (int)fns.size();
  std::vector<int> atom0(nf, 0), lxyz(3 * nf), nprim(nf);
  std::vector<double> coef, expo;
  for (int k = 0; k < nf; ++k) {
    const int i = fns[k];
    for (int x = 0; x < 3; ++x) lxyz[3 * k + x] = b.cgf_lxyz[3 * i + x];
    nprim[k] = b.cgf_nprim[i];
    for (int p = b.cgf_off[i]; p < b.cgf_off[i + 1]; ++p) {
      coef.push_back(b.prim_coef[p]);
      expo.push_back(b.prim_exp[p]);
    }
  }
  const double origin[3] = {0, 0, 0};
  const double Z = b.Z[a];
  GBHF_TRY(build_basis(sub, 1, origin, &Z, nf, atom0.data(), lxyz.data(), nprim.data(), coef.data(), expo.data()));
  if (sub->basis.maxL > 2) return fail(c, GBHF_ERR_UNSUPPORTED, "SAD guess: atomic basis above d functions");
  GBHF_TRY(ensure_boys_tables(sub));
  const int n = nf;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  GBHF_WS(sub, fS, 0, ntri);
  GBHF_WS(sub, fH, 1, ntri);
  GBHF_WS(sub, fD, 2, ntri);
  GBHF_WS(sub, fF, 3, ntri);
  GBHF_WS(sub, S, 4, nn);
  GBHF_WS(sub, X, 5, nn);
  GBHF_WS(sub, F, 6, nn);
  GBHF_WS(sub, T, 7, nn);
  GBHF_WS(sub, C, 8, nn);
  GBHF_WS(sub, Dm, 9, nn);
  GBHF_WS(sub, Dn, 15, nn);
  GBHF_WS(sub, eps, 16, n);
  GBHF_WS(sub, occd, 17, n);
  GBHF_WS(sub, Cp, 18, nn);
  GBHF_TRY(onee_matrices(sub, false, fS, fH));
  GBHF_TRY(flat_to_square(sub, n, fS, S));
  GBHF_TRY(symm_ortho_dev(sub, n, S, X));
  const long long P = (long long)ntri;
  DBuf<double> eri;
  GBHF_CUDA(c, eri.alloc((size_t)(P * (P + 1) / 2)));
  GBHF_TRY(eri_canonical_dev(sub, false, eri.p));
  GBHF_TRY(flat_to_square(sub, n, fH, F));
  std::vector<double> h_eps(n), occ;
  bool have_d = false;
  for (int it = 0; it < 200; ++it) {
    // orbitals of F: F' = X^T F X, C = X C'
    GBHF_TRY(gemm(sub, true, false, n, n, n, 1.0, X, n, F, n, 0.0, T, n));
    GBHF_TRY(gemm(sub, false, false, n, n, n, 1.0, T, n, X, n, 0.0, Cp, n));
    GBHF_TRY(eigh(sub, n, Cp, eps, T, nullptr));
    GBHF_TRY(gemm(sub, false, false, n, n, n, 1.0, X, n, T, n, 0.0, C, n));
    GBHF_CUDA(c, cudaMemcpyAsync(h_eps.data(), eps, n * sizeof(double), cudaMemcpyDeviceToHost, sub->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(sub->stream));
    frac_occupations(h_eps, Z, occ);
    GBHF_CUDA(c, cudaMemcpyAsync(occd, occ.data(), n * sizeof(double), cudaMemcpyHostToDevice, sub->stream));
    k_sad_scale_cols<<<dim3((n + 127) / 128, n), 128, 0, sub->stream>>>(n, C, occd, T);
    count_launch(sub);
    GBHF_CUDA(c, cudaGetLastError());
    GBHF_TRY(gemm(sub, false, true, n, n, n, 1.0, T, n, C, n, 0.0, Dn, n));
    double change = 1.0;
    if (have_d) {
      GBHF_TRY(axpby(sub, nn, 1.0, Dn, -1.0, Dm, T));
      GBHF_TRY(max_abs(sub, nn, T, &change));
    }
    // damped for the first steps, then plain Roothaan steps
    if (have_d && it < 4) GBHF_TRY(axpby(sub, nn, 0.5, Dn, 0.5, Dm, Dm));
    else GBHF_CUDA(c, cudaMemcpyAsync(Dm, Dn, nn * sizeof(double), cudaMemcpyDeviceToDevice, sub->stream));
    have_d = true;
    if (change < 1e-10) break;
    GBHF_TRY(square_to_flat(sub, n, Dm, fD));
    GBHF_TRY(fock_canonical_dev(sub, fH, fD, eri.p, fF));
    GBHF_TRY(flat_to_square(sub, n, fF, F));
  }
  block.resize(nn);
  GBHF_CUDA(c, cudaMemcpyAsync(block.data(), Dm, nn * sizeof(double), cudaMemcpyDeviceToHost, sub->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(sub->stream));
  return GBHF_OK;
}

// Atomic density blocks by atom key (element and its contracted functions):
// shared by the contexts of the process, so that a new context (e.g. one per
// call of a host that creates and destroys one) does not rerun the atomic SCFs.
static std::mutex g_sad_mu;
static std::map<std::string, std::vector<double>> g_sad_cache;

// Stacked blocks of every molecule of the context's basis (one block for one molecule).
gbhf_status sad_density(gbhf_ctx* c, double* d_D) {
  const Basis& b = c->basis;
  const int n = b.nbf;
  std::vector<int> fatom(n), floc(n), boff(b.natoms), bdim(b.natoms);
  std::vector<double> blocks;
  std::vector<int> fns;
  for (int a = 0; a < b.natoms; ++a) {
    const std::string key = atom_key(b, a, fns);
    auto it = c->sad_cache.find(key);
    if (it == c->sad_cache.end()) {
      std::lock_guard<std::mutex> lock(g_sad_mu);
      auto g = g_sad_cache.find(key);
      if (g != g_sad_cache.end()) it = c->sad_cache.emplace(key, g->second).first;
    }
    if (it == c->sad_cache.end()) {
      if (!c->sad_ctx) {
        gbhf_ctx* sub = nullptr;
        if (gbhf_create(&sub, c->device) != GBHF_OK) return fail(c, GBHF_ERR_CUDA, "SAD guess: context creation failed");
        c->sad_ctx = sub;
        cudaSetDevice(c->device);
      }
      std::vector<double> blk;
      const gbhf_status s = atomic_density(c, c->sad_ctx, b, a, fns, blk);
      if (s != GBHF_OK) {
        if (!c->sad_ctx->err.empty()) c->err = "SAD guess: " + c->sad_ctx->err;
        return s;
      }
      {
        std::lock_guard<std::mutex> lock(g_sad_mu);
        g_sad_cache.emplace(key, blk);
      }
      it = c->sad_cache.emplace(key, std::move(blk)).first;
    }
    boff[a] = (int)blocks.size();
    bdim[a] = (int)fns.size();
    blocks.insert(blocks.end(), it->second.begin(), it->second.end());
    for (int k = 0; k < (int)fns.size(); ++k) {
      fatom[fns[k]] = a;
      floc[fns[k]] = k;
    }
  }
  DBuf<int> dfa, dfl, dbo, dbd;
  DBuf<double> dbl;
  GBHF_CUDA(c, dfa.alloc(n));
  GBHF_CUDA(c, dfl.alloc(n));
  GBHF_CUDA(c, dbo.alloc(b.natoms));
  GBHF_CUDA(c, dbd.alloc(b.natoms));
  GBHF_CUDA(c, dbl.alloc(std::max<size_t>(blocks.size(), 1)));
  GBHF_CUDA(c, cudaMemcpyAsync(dfa.p, fatom.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dfl.p, floc.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dbo.p, boff.data(), b.natoms * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dbd.p, bdim.data(), b.natoms * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(dbl.p, blocks.data(), blocks.size() * sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
  GBHF_TRY(ensure_shell_arrays(c));
  int max_fn = 0;
  for (int m = 0; m < b.nmol; ++m) max_fn = std::max(max_fn, b.mol_fn_off[m + 1] - b.mol_fn_off[m]);
  k_sad_assemble<<<dim3((max_fn + 127) / 128, n), 128, 0, c->stream>>>(
      c->tasks.fmol.p, c->tasks.mfo.p, c->tasks.moff.p, dfa.p, dfl.p, dbo.p, dbd.p, dbl.p, d_D);
  count_launch(c);
  GBHF_CUDA(c, cudaGetLastError());
  // the staging buffers are freed on return: finish the copies and the kernel
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

}  // namespace gbhf
