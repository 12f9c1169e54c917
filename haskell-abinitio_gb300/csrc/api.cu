// C ABI of libgbhf (declarations and reference citations in include/gbhf.h).
#include <cstdlib>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gbhf_internal.h"

using namespace gbhf;

namespace {

gbhf_status check_ctx(gbhf_ctx* c) {
  if (!c) return GBHF_ERR_BAD_INPUT;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  return GBHF_OK;
}

#define CTX_CHECK(c)                            \
  gbhf::PoolScope pool_scope__(c);              \
  do {                                          \
    if (!(c)) return GBHF_ERR_BAD_INPUT;        \
    gbhf_status s0__ = check_ctx(c);            \
    if (s0__ != GBHF_OK) return s0__;           \
    (c)->err.clear();                           \
  } while (0)

template <typename T>
gbhf_status upload(gbhf_ctx* c, DBuf<T>& d, const T* h, size_t n) {
  GBHF_CUDA(c, d.alloc(n));
  GBHF_CUDA(c, cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  return GBHF_OK;
}

gbhf_status download(gbhf_ctx* c, void* h, const void* d, size_t bytes) {
  GBHF_CUDA(c, cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c->stream));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

bool need_basis(gbhf_ctx* c) {
  if (!c->basis_dev) {
    c->err = "no basis set (call gbhf_set_basis first)";
    return false;
  }
  if (c->basis.nmol != 1) {
    c->err = "the context holds the basis of a batch (call gbhf_set_basis first)";
    return false;
  }
  return true;
}

}  // namespace

extern "C" {

int gbhf_version(void) { return 1; }

gbhf_status gbhf_create(gbhf_ctx** out, int device) {
  if (!out) return GBHF_ERR_BAD_INPUT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return GBHF_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return GBHF_ERR_NO_DEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return GBHF_ERR_NO_DEVICE;
  gbhf_ctx* c = new gbhf_ctx;
  c->device = device;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    delete c;
    return GBHF_ERR_NO_DEVICE;
  }
  c->nsm = prop.multiProcessorCount;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  {
    const char* ev = std::getenv("GBHF_EIGEN");
    c->force_jacobi = ev && std::string(ev) == "jacobi";
    c->force_sytrd_single = ev && std::string(ev) == "single-cta";
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return GBHF_ERR_CUDA;
  }
  for (auto& e : c->ev) cudaEventCreate(&e);
  for (auto& e : c->evc) cudaEventCreate(&e);
  for (auto& e : c->evu) cudaEventCreate(&e);
  for (auto& e : c->evg) cudaEventCreate(&e);
  for (auto& e : c->evp) cudaEventCreate(&e);
  default_budgets(c, 0);
  default_budgets(c, 1);
  for (int i = 0; i < gbhf_ctx::NSIDE; ++i) {
    if (cudaStreamCreateWithFlags(&c->side[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join_ev[i], cudaEventDisableTiming) != cudaSuccess) {
      gbhf_destroy(c);
      return GBHF_ERR_CUDA;
    }
  }
  if (cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess) {
    gbhf_destroy(c);
    return GBHF_ERR_CUDA;
  }
  *out = c;
  return GBHF_OK;
}

gbhf_status gbhf_destroy(gbhf_ctx* c) {
  if (!c) return GBHF_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->evc)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->evu)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->evg)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->evp)
    if (e) cudaEventDestroy(e);
  for (int i = 0; i < gbhf_ctx::NSIDE; ++i) {
    if (c->side[i]) {
      cudaStreamSynchronize(c->side[i]);
      cudaStreamDestroy(c->side[i]);
    }
    if (c->join_ev[i]) cudaEventDestroy(c->join_ev[i]);
  }
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  for (gbhf_ctx* w : c->pool) gbhf_destroy(w);
  c->pool.clear();
  if (c->sad_ctx) gbhf_destroy(c->sad_ctx);
  c->sad_ctx = nullptr;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  delete c;   // frees device buffers
  if (s) cudaStreamDestroy(s);
  return GBHF_OK;
}

const char* gbhf_last_error(gbhf_ctx* c) { return c ? c->err.c_str() : "null context"; }

gbhf_status gbhf_set_basis(gbhf_ctx* c, int n_atoms, const double* xyz, const double* Z, int n_cgf,
                           const int* cgf_atom, const int* cgf_lxyz, const int* cgf_nprim, const double* coef,
                           const double* expo) {
  CTX_CHECK(c);
  c->tasks.thr_all = -1;
  c->tasks.thr64 = -1;
  return build_basis(c, n_atoms, xyz, Z, n_cgf, cgf_atom, cgf_lxyz, cgf_nprim, coef, expo);
}

gbhf_status gbhf_set_boys_grid(gbhf_ctx* c, const double* grid) {
  CTX_CHECK(c);
  if (!grid) return fail(c, GBHF_ERR_BAD_INPUT, "null grid");
  for (int i = 0; i < 15 * 1001; ++i)
    if (!std::isfinite(grid[i])) return fail(c, GBHF_ERR_BAD_INPUT, "Boys grid holds a non-finite value");
  GBHF_TRY(upload(c, c->boys_ref, grid, 15 * 1001));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_grid = true;
  return GBHF_OK;
}

gbhf_status gbhf_generate_boys_grid(gbhf_ctx* c, double* grid_out) {
  CTX_CHECK(c);
  GBHF_CUDA(c, c->boys_ref.alloc(15 * 1001));
  GBHF_TRY(boys_ref_grid_dev(c, c->boys_ref.p));
  c->have_grid = true;
  if (grid_out) return download(c, grid_out, c->boys_ref.p, 15 * 1001 * sizeof(double));
  return GBHF_OK;
}

gbhf_status gbhf_boys(gbhf_ctx* c, int mode, int m_max, int n, const double* x, double* out) {
  CTX_CHECK(c);
  if (n < 0 || (n > 0 && (!x || !out))) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_boys: bad arguments");
  const bool ref = mode == GBHF_MODE_REFERENCE;
  if (ref && !c->have_grid) return fail(c, GBHF_ERR_BAD_INPUT, "reference mode needs gbhf_set_boys_grid");
  for (int i = 0; i < n; ++i)
    if (!(x[i] >= 0) || !std::isfinite(x[i])) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_boys: x must be finite, >= 0");
  GBHF_TRY(ensure_boys_tables(c));
  if (n == 0) return GBHF_OK;
  DBuf<double> dx, dout;
  GBHF_TRY(upload(c, dx, x, n));
  GBHF_CUDA(c, dout.alloc((size_t)n * (m_max + 1)));
  GBHF_TRY(boys_dev(c, ref, m_max, n, dx.p, dout.p));
  return download(c, out, dout.p, (size_t)n * (m_max + 1) * sizeof(double));
}

gbhf_status gbhf_overlap(gbhf_ctx* c, int mode, double* s_flat) {
  CTX_CHECK(c);
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  if (!s_flat) return fail(c, GBHF_ERR_BAD_INPUT, "null output");
  GBHF_TRY(ensure_boys_tables(c));
  const size_t ntri = (size_t)c->basis.nbf * (c->basis.nbf + 1) / 2;
  GBHF_WS(c, d, 15, ntri);
  GBHF_TRY(onee_matrices(c, mode == GBHF_MODE_REFERENCE, d, nullptr));
  return download(c, s_flat, d, ntri * sizeof(double));
}

gbhf_status gbhf_hcore(gbhf_ctx* c, int mode, double* h_flat) {
  CTX_CHECK(c);
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  if (!h_flat) return fail(c, GBHF_ERR_BAD_INPUT, "null output");
  GBHF_TRY(ensure_boys_tables(c));
  const size_t ntri = (size_t)c->basis.nbf * (c->basis.nbf + 1) / 2;
  GBHF_WS(c, d, 16, ntri);
  GBHF_TRY(onee_matrices(c, mode == GBHF_MODE_REFERENCE, nullptr, d));
  return download(c, h_flat, d, ntri * sizeof(double));
}

int64_t gbhf_eri_canonical_length(int n) {
  if (n <= 0) return 0;
  const int64_t p = (int64_t)n * (n + 1) / 2;
  return p * (p + 1) / 2;
}

gbhf_status gbhf_eri_canonical(gbhf_ctx* c, int mode, double* eri, int64_t length) {
  CTX_CHECK(c);
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  const int64_t need = gbhf_eri_canonical_length(c->basis.nbf);
  if (!eri || length < need) return fail(c, GBHF_ERR_BAD_INPUT, "ERI output buffer too small");
  GBHF_TRY(ensure_boys_tables(c));
  DBuf<double> d;
  GBHF_CUDA(c, d.alloc((size_t)need));
  GBHF_TRY(eri_canonical_dev(c, mode == GBHF_MODE_REFERENCE, d.p));
  return download(c, eri, d.p, (size_t)need * sizeof(double));
}

gbhf_status gbhf_fock(gbhf_ctx* c, int mode, int precision, double schwarz_cutoff, double mixed_cutoff,
                      const double* h_flat, const double* d_flat, double* f_flat) {
  CTX_CHECK(c);
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  if (!h_flat || !d_flat || !f_flat) return fail(c, GBHF_ERR_BAD_INPUT, "null pointer");
  if (!(schwarz_cutoff >= 0) || !(mixed_cutoff >= 0)) return fail(c, GBHF_ERR_BAD_INPUT, "cutoffs must be >= 0");
  GBHF_TRY(ensure_boys_tables(c));
  const int n = c->basis.nbf;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  GBHF_WS(c, fH, 15, ntri);
  GBHF_WS(c, fD, 16, ntri);
  GBHF_WS(c, fF, 17, ntri);
  GBHF_CUDA(c, cudaMemcpyAsync(fH, h_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(fD, d_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (mode == GBHF_MODE_REFERENCE) {
    if (!c->have_grid) return fail(c, GBHF_ERR_BAD_INPUT, "reference mode needs gbhf_set_boys_grid");
    const long long P = (long long)ntri;
    DBuf<double> eri;
    GBHF_CUDA(c, eri.alloc((size_t)(P * (P + 1) / 2)));
    GBHF_TRY(eri_canonical_dev(c, true, eri.p));
    GBHF_TRY(fock_canonical_dev(c, fH, fD, eri.p, fF));
    return download(c, f_flat, fF, ntri * sizeof(double));
  }
  GBHF_WS(c, Dsq, 18, nn);
  GBHF_WS(c, Hsq, 19, nn);
  GBHF_WS(c, Gpp, 20, nn);
  GBHF_WS(c, Fsq, 21, nn);
  GBHF_TRY(flat_to_square(c, n, fD, Dsq));
  GBHF_TRY(flat_to_square(c, n, fH, Hsq));
  GBHF_CUDA(c, cudaMemsetAsync(Gpp, 0, nn * sizeof(double), c->stream));
  GBHF_TRY(jk_build(c, Dsq, Gpp, precision, schwarz_cutoff, mixed_cutoff, 1.0));
  GBHF_TRY(add_sym(c, n, Hsq, Gpp, Fsq));
  GBHF_TRY(square_to_flat(c, n, Fsq, fF));
  return download(c, f_flat, fF, ntri * sizeof(double));
}

gbhf_status gbhf_symm_ortho(gbhf_ctx* c, int n, const double* s_square, double* x_square) {
  CTX_CHECK(c);
  if (n <= 0 || !s_square || !x_square) return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, S, 15, nn);
  GBHF_WS(c, X, 16, nn);
  GBHF_CUDA(c, cudaMemcpyAsync(S, s_square, nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(symm_ortho_dev(c, n, S, X));
  return download(c, x_square, X, nn * sizeof(double));
}

gbhf_status gbhf_eigen_solve(gbhf_ctx* c, int n, const double* a_square, double* evals, double* evecs) {
  CTX_CHECK(c);
  if (n <= 0 || !a_square || !evals || !evecs) return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  const size_t nn = (size_t)n * n;
  GBHF_WS(c, A, 15, nn);
  GBHF_WS(c, V, 16, nn);
  GBHF_WS(c, w, 17, (size_t)n);
  GBHF_CUDA(c, cudaMemcpyAsync(A, a_square, nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(eigh(c, n, A, w, V, nullptr));
  GBHF_TRY(download(c, evals, w, n * sizeof(double)));
  return download(c, evecs, V, nn * sizeof(double));
}

gbhf_status gbhf_sad_density(gbhf_ctx* c, double* density_flat) {
  CTX_CHECK(c);
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  if (!density_flat) return fail(c, GBHF_ERR_BAD_INPUT, "null output");
  const int n = c->basis.nbf;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  GBHF_WS(c, Dsq, 15, nn);
  GBHF_WS(c, fD, 16, ntri);
  GBHF_TRY(sad_density(c, Dsq));
  GBHF_TRY(square_to_flat(c, n, Dsq, fD));
  GBHF_TRY(download(c, density_flat, fD, ntri * sizeof(double)));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

gbhf_status gbhf_diagonal_hf(gbhf_ctx* c, int n, const double* f_flat, const double* x_square, int n_occupied,
                             double* coeff, double* density_flat, double* orb_energies) {
  CTX_CHECK(c);
  if (n <= 0 || !f_flat || !x_square || n_occupied < 0 || n_occupied > n)
    return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  GBHF_WS(c, fF, 15, ntri);
  GBHF_WS(c, Fsq, 16, nn);
  GBHF_WS(c, X, 17, nn);
  GBHF_WS(c, C, 18, nn);
  GBHF_WS(c, Dsq, 19, nn);
  GBHF_WS(c, eps, 20, (size_t)n);
  GBHF_WS(c, fD, 21, ntri);
  GBHF_CUDA(c, cudaMemcpyAsync(fF, f_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(X, x_square, nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(flat_to_square(c, n, fF, Fsq));
  GBHF_TRY(diagonal_hf_dev(c, n, Fsq, X, n_occupied, C, Dsq, eps, nullptr));
  GBHF_TRY(square_to_flat(c, n, Dsq, fD));
  if (coeff) GBHF_TRY(download(c, coeff, C, nn * sizeof(double)));
  if (density_flat) GBHF_TRY(download(c, density_flat, fD, ntri * sizeof(double)));
  if (orb_energies) GBHF_TRY(download(c, orb_energies, eps, n * sizeof(double)));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

gbhf_status gbhf_diis_error(gbhf_ctx* c, int n, const double* f_flat, const double* s_flat, const double* d_flat,
                            const double* x_square, double* e_square) {
  CTX_CHECK(c);
  if (n <= 0 || !f_flat || !s_flat || !d_flat || !x_square || !e_square)
    return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  GBHF_WS(c, t, 15, ntri);
  GBHF_WS(c, F, 16, nn);
  GBHF_WS(c, S, 17, nn);
  GBHF_WS(c, D, 18, nn);
  GBHF_WS(c, X, 19, nn);
  GBHF_WS(c, E, 20, nn);
  GBHF_CUDA(c, cudaMemcpyAsync(t, f_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(flat_to_square(c, n, t, F));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(t, s_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(flat_to_square(c, n, t, S));
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(t, d_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(flat_to_square(c, n, t, D));
  GBHF_CUDA(c, cudaMemcpyAsync(X, x_square, nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GBHF_TRY(diis_error_dev(c, n, F, S, D, X, E));
  return download(c, e_square, E, nn * sizeof(double));
}

gbhf_status gbhf_gauss_elem(gbhf_ctx* c, int m, const double* a, const double* b, double* x) {
  CTX_CHECK(c);
  if (!a || !b || !x) return fail(c, GBHF_ERR_BAD_INPUT, "null pointer");
  bool ok = false;
  GBHF_TRY(gauss_elem_dev_call(c, m, a, b, x, &ok));
  if (!ok) return fail(c, GBHF_ERR_SINGULAR, "Gauss elimination: rank deficient or non-finite system");
  return GBHF_OK;
}

gbhf_status gbhf_diis_extrapolate(gbhf_ctx* c, int n, int n_hist, const double* errors_square,
                                  const double* focks_flat, double* f_out_flat, int* n_used) {
  CTX_CHECK(c);
  if (n <= 0 || n_hist < 0 || n_hist > 7 || !errors_square || !focks_flat || !f_out_flat)
    return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  const int k0 = n_hist + 1;
  DBuf<double> E, Fv, out, dots;
  GBHF_TRY(upload(c, E, errors_square, nn * k0));
  GBHF_TRY(upload(c, Fv, focks_flat, ntri * k0));
  GBHF_CUDA(c, out.alloc(ntri));
  GBHF_CUDA(c, dots.alloc(64));
  // B_ij = tr(e_i^T e_j)
  std::vector<double> B((size_t)k0 * k0);
  for (int i = 0; i < k0; ++i) {
    std::vector<const double*> mats;
    for (int j = 0; j < k0; ++j) mats.push_back(E.p + nn * j);
    GBHF_TRY(dot_matrices(c, (int)nn, k0, mats.data(), E.p + nn * i, dots.p));
    GBHF_TRY(download(c, &B[(size_t)i * k0], dots.p, k0 * sizeof(double)));
  }
  int k = k0;
  while (true) {
    const int m = k + 1;
    std::vector<double> Bm((size_t)m * m, 0.0), rhs(m, 0.0), x(m, 0.0);
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) Bm[(size_t)i * m + j] = B[(size_t)i * k0 + j];
    for (int i = 0; i < k; ++i) {
      Bm[(size_t)i * m + k] = -1;
      Bm[(size_t)k * m + i] = -1;
    }
    rhs[k] = -1;
    bool ok = false;
    GBHF_TRY(gauss_elem_dev_call(c, m, Bm.data(), rhs.data(), x.data(), &ok));
    if (ok) {
      std::vector<const double*> mats;
      for (int j = 0; j < k; ++j) mats.push_back(Fv.p + ntri * j);
      GBHF_CUDA(c, cudaMemcpyAsync(dots.p, x.data(), k * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      GBHF_TRY(lincomb(c, (int)ntri, k, mats.data(), dots.p, out.p));
      if (n_used) *n_used = k - 1;
      return download(c, f_out_flat, out.p, ntri * sizeof(double));
    }
    if (k == 1) return fail(c, GBHF_ERR_SINGULAR, "DIIS system singular with no stored vectors left");
    --k;
  }
}

void gbhf_scf_opts_reference(gbhf_scf_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->mode = GBHF_MODE_REFERENCE;
  o->precision = GBHF_PREC_FP64;
  o->guess = GBHF_GUESS_HARRIS;
  o->diis_size = 5;
  o->max_iter = 30;
  o->incremental = 0;
  o->full_rebuild_every = 0;
  o->final_fp64 = 0;
  o->ref_stop_rule = 1;
  o->conv_error = 1e-7;
  o->conv_energy = 1e-10;
  o->conv_density = 1e-8;
  o->diis_start = 0.1;
  o->schwarz_cutoff = 0.0;
  o->mixed_cutoff = 0.0;
  o->charge = 0.0;
}

void gbhf_scf_opts_baseline(gbhf_scf_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->mode = GBHF_MODE_EXACT;
  o->precision = GBHF_PREC_FP64;
  o->guess = GBHF_GUESS_SAD;
  o->diis_size = 6;
  o->max_iter = 100;
  o->incremental = 0;
  o->full_rebuild_every = 8;
  o->final_fp64 = 1;
  o->ref_stop_rule = 0;
  o->conv_error = 1e-7;
  o->conv_energy = 1e-10;
  o->conv_density = 1e-8;
  o->diis_start = 1e30;
  o->schwarz_cutoff = 1e-12;
  o->mixed_cutoff = 1e-4;
  o->charge = 0.0;
}

gbhf_status gbhf_scf(gbhf_ctx* c, const gbhf_scf_opts* opts, gbhf_result* result) {
  CTX_CHECK(c);
  if (!opts) return fail(c, GBHF_ERR_BAD_INPUT, "null options");
  return scf_run(c, opts, result);
}

gbhf_status gbhf_scf_uhf(gbhf_ctx* c, const gbhf_scf_opts* opts, int multiplicity, gbhf_uhf_result* result) {
  CTX_CHECK(c);
  if (!opts) return fail(c, GBHF_ERR_BAD_INPUT, "null options");
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  return uhf_run(c, opts, multiplicity, result);
}

gbhf_status gbhf_gradient(gbhf_ctx* c, int precision, double schwarz_cutoff, const double* d_flat,
                          const double* w_flat, double* grad) {
  CTX_CHECK(c);
  if (precision != GBHF_PREC_FP64 && precision != GBHF_PREC_MIXED)
    return fail(c, GBHF_ERR_BAD_INPUT, "precision must be GBHF_PREC_FP64 or GBHF_PREC_MIXED");
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  if (!grad || !(schwarz_cutoff >= 0)) return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  if ((d_flat == nullptr) != (w_flat == nullptr))
    return fail(c, GBHF_ERR_BAD_INPUT, "give both D and W, or neither (use the last SCF)");
  const int n = c->basis.nbf, na = c->basis.natoms;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  GBHF_WS(c, D, 15, nn);
  GBHF_WS(c, W, 16, nn);
  GBHF_WS(c, t, 17, std::max(ntri, (size_t)n));
  if (d_flat) {
    GBHF_CUDA(c, cudaMemcpyAsync(t, d_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    GBHF_TRY(flat_to_square(c, n, t, D));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(t, w_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    GBHF_TRY(flat_to_square(c, n, t, W));
  } else {
    if (c->last_gen != c->basis_gen || c->last_nocc < 0)
      return fail(c, GBHF_ERR_BAD_INPUT, "no converged SCF for this basis: run gbhf_scf first or pass D and W");
    // orbitals of the converged Fock matrix -> W; D from the SCF
    GBHF_WS(c, S, 18, nn);
    GBHF_WS(c, X, 19, nn);
    GBHF_WS(c, Cm, 20, nn);
    GBHF_WS(c, Dt, 21, nn);
    GBHF_TRY(onee_matrices(c, false, t, nullptr));
    GBHF_TRY(flat_to_square(c, n, t, S));
    int it = 0;
    GBHF_TRY(inv_sqrt_dev(c, n, S, X, &it));
    GBHF_WS(c, eps, 22, (size_t)n);
    GBHF_TRY(diagonal_hf_dev(c, n, c->last_F.p, X, c->last_nocc, Cm, Dt, eps, nullptr));
    GBHF_TRY(energy_weighted_density(c, n, c->last_nocc, Cm, eps, W));
    // D and W from the same orbitals
    GBHF_CUDA(c, cudaMemcpyAsync(D, Dt, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  }
  DBuf<double> g;
  GBHF_CUDA(c, g.alloc(3 * (size_t)na));
  // mixed precision: FP32 derivative integrals for quartets whose bound
  // Q_ab Q_cd max(w)^2 is below 1e-4, the SCF's mixed cutoff
  GBHF_TRY(gradient_dev(c, D, W, schwarz_cutoff, 1e-4, precision, g.p));
  return download(c, grad, g.p, 3 * (size_t)na * sizeof(double));
}

gbhf_status gbhf_gradient_uhf(gbhf_ctx* c, int precision, double schwarz_cutoff, const double* da_flat,
                              const double* db_flat, const double* w_flat, double* grad) {
  CTX_CHECK(c);
  if (precision != GBHF_PREC_FP64 && precision != GBHF_PREC_MIXED)
    return fail(c, GBHF_ERR_BAD_INPUT, "precision must be GBHF_PREC_FP64 or GBHF_PREC_MIXED");
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  if (!grad || !(schwarz_cutoff >= 0)) return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  const bool given = da_flat || db_flat || w_flat;
  if (given && !(da_flat && db_flat && w_flat))
    return fail(c, GBHF_ERR_BAD_INPUT, "give D_alpha, D_beta and W, or none (use the last UHF SCF)");
  const int n = c->basis.nbf, na = c->basis.natoms;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  const double *Da = nullptr, *Db = nullptr, *W = nullptr;
  GBHF_WS(c, Sa, 15, nn);
  GBHF_WS(c, Sb, 16, nn);
  GBHF_WS(c, Sw, 18, nn);
  GBHF_WS(c, t, 17, std::max(ntri, (size_t)n));
  if (given) {
    const double* src[3] = {da_flat, db_flat, w_flat};
    double* dst[3] = {Sa, Sb, Sw};
    for (int k = 0; k < 3; ++k) {
      GBHF_CUDA(c, cudaMemcpyAsync(t, src[k], ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      GBHF_TRY(flat_to_square(c, n, t, dst[k]));
      GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    Da = Sa;
    Db = Sb;
    W = Sw;
  } else {
    if (c->last_ugen != c->basis_gen || !c->last_uDa.p)
      return fail(c, GBHF_ERR_BAD_INPUT, "no converged UHF SCF for this basis: run gbhf_scf_uhf first or pass the densities");
    Da = c->last_uDa.p;
    Db = c->last_uDb.p;
    W = c->last_uW.p;
  }
  DBuf<double> g;
  GBHF_CUDA(c, g.alloc(3 * (size_t)na));
  GBHF_TRY(gradient_uhf_dev(c, Da, Db, W, schwarz_cutoff, 1e-4, precision, g.p));
  return download(c, grad, g.p, 3 * (size_t)na * sizeof(double));
}

static int budget_classes(int which) { return which == 0 ? NCOMBO : which == 1 ? NCOMBO_MAX : 0; }

gbhf_status gbhf_get_task_budgets(gbhf_ctx* c, int which, int* budgets, int n) {
  CTX_CHECK(c);
  const int nc = budget_classes(which);
  if (nc == 0 || !budgets || n < 2 * nc) return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  const int* lp = which == 0 ? c->jk_lp : c->gr_lp;
  const int* tk = which == 0 ? c->jk_tk : c->gr_tk;
  for (int k = 0; k < nc; ++k) {
    budgets[2 * k] = lp[k];
    budgets[2 * k + 1] = tk[k];
  }
  return GBHF_OK;
}

gbhf_status gbhf_set_task_budgets(gbhf_ctx* c, int which, const int* budgets, int n) {
  CTX_CHECK(c);
  const int nc = budget_classes(which);
  if (nc == 0 || n < 2 * nc) return fail(c, GBHF_ERR_BAD_INPUT, "bad arguments");
  if (!budgets) {   // back to the defaults
    default_budgets(c, which);
    c->tuned[which] = false;
  } else {
    for (int k = 0; k < nc; ++k)
      if (budgets[2 * k] < 1 || budgets[2 * k] > 65535 || budgets[2 * k + 1] < 1 || budgets[2 * k + 1] > 32)
        return fail(c, GBHF_ERR_BAD_INPUT, "budgets: primitive quartets per lane 1..65535, kets per task 1..32");
    int* lp = which == 0 ? c->jk_lp : c->gr_lp;
    int* tk = which == 0 ? c->jk_tk : c->gr_tk;
    for (int k = 0; k < nc; ++k) {
      lp[k] = budgets[2 * k];
      tk[k] = budgets[2 * k + 1];
    }
    c->tuned[which] = true;
  }
  if (which == 0) c->tasks.thr_all = -1;   // cached lists follow the old budgets
  return GBHF_OK;
}

gbhf_status gbhf_autotune(gbhf_ctx* c, int which, int precision, double schwarz_cutoff, double mixed_cutoff,
                          const double* density_flat, int repeats, double* class_ms) {
  CTX_CHECK(c);
  if (budget_classes(which) == 0) return fail(c, GBHF_ERR_BAD_INPUT, "which must be 0 (J/K) or 1 (gradient)");
  if (precision != GBHF_PREC_FP64 && precision != GBHF_PREC_MIXED)
    return fail(c, GBHF_ERR_BAD_INPUT, "precision must be GBHF_PREC_FP64 or GBHF_PREC_MIXED");
  if (!(schwarz_cutoff >= 0) || !(mixed_cutoff >= 0) || repeats < 1)
    return fail(c, GBHF_ERR_BAD_INPUT, "cutoffs must be >= 0 and repeats >= 1");
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  const Basis& b = c->basis;
  if (!b.shells_ok || b.maxL > 2) return fail(c, GBHF_ERR_UNSUPPORTED, "direct builds need complete s, p, d shells");
  GBHF_TRY(ensure_boys_tables(c));
  GBHF_TRY(ensure_pairs(c));
  GBHF_TRY(ensure_shell_arrays(c));
  const int n = b.nbf;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  GBHF_WS(c, D, 15, nn);
  if (density_flat) {
    GBHF_WS(c, t, 16, ntri);
    GBHF_CUDA(c, cudaMemcpyAsync(t, density_flat, ntri * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    GBHF_TRY(flat_to_square(c, n, t, D));
  } else {
    GBHF_TRY(sad_density(c, D));
  }
  const double mc = precision == GBHF_PREC_FP64 ? 0.0 : mixed_cutoff;
  return autotune_dev(c, which, D, precision, schwarz_cutoff, mc, repeats, class_ms);
}

gbhf_status gbhf_profile_reset(gbhf_ctx* c, int enable_events) {
  CTX_CHECK(c);
  GBHF_TRY(flush_jk_stats(c));   // counts of earlier builds go with the old profile
  c->prof = Profile();
  c->prof.events = enable_events != 0;
  return GBHF_OK;
}

gbhf_status gbhf_set_guess_density(gbhf_ctx* c, const double* density_flat) {
  CTX_CHECK(c);
  if (!need_basis(c)) return GBHF_ERR_BAD_INPUT;
  if (!density_flat) return fail(c, GBHF_ERR_BAD_INPUT, "null density");
  const size_t n = (size_t)c->basis.nbf;
  GBHF_TRY(upload(c, c->guess_D, density_flat, n * (n + 1) / 2));
  c->guess_gen = c->basis_gen;
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

gbhf_status gbhf_scf_trace(gbhf_ctx* c, double* out, int max_records, int* n_records) {
  CTX_CHECK(c);
  if (!n_records || (max_records > 0 && !out)) return fail(c, GBHF_ERR_BAD_INPUT, "null pointer");
  const int nrec = (int)(c->scf_trace.size() / GBHF_SCF_TRACE_FIELDS);
  *n_records = nrec;
  const int m = std::min(nrec, std::max(max_records, 0));
  std::copy(c->scf_trace.begin(), c->scf_trace.begin() + (size_t)m * GBHF_SCF_TRACE_FIELDS, out);
  return GBHF_OK;
}

gbhf_status gbhf_profile_read(gbhf_ctx* c, double* stats, int n_stats) {
  CTX_CHECK(c);
  if (!stats) return fail(c, GBHF_ERR_BAD_INPUT, "null pointer");
  GBHF_TRY(flush_jk_stats(c));
  const double v[20] = {c->prof.jk_ms64,   c->prof.jk_ms32,  c->prof.prim64,        c->prof.prim32,
                        c->prof.shellq,    c->prof.fnq,      (double)c->prof.launches, c->prof.dense_ms,
                        c->prof.ph_setup,  c->prof.ph_fock,  c->prof.ph_diis,       c->prof.ph_diag,
                        c->prof.ph_other,  c->prof.jacobi_sweeps, c->prof.jacobi_calls, c->prof.ph_grad,
                        c->prof.batch_steps, c->prof.purify_steps, c->prof.purify_calls, c->prof.ph_pairs};
  for (int i = 0; i < n_stats && i < 20; ++i) stats[i] = v[i];
  return GBHF_OK;
}

}  // extern "C"
