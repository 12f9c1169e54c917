// SCF driver (scfHF / scfDIIS, HartreeFock/HartreeFock.hs:70-123) on the device.
// Every matrix lives in HBM; per iteration the host reads back a handful of
// scalars (max|e|, energy, RMS dD, DIIS dot products) to take the branch
// decisions of the reference driver.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbhf_internal.h"

namespace gbhf {

// Literal fourIndex2Flat (NumericalTools/LinearAlgebra.hs:266-283) for any n,
// as the Harris guess (HartreeFock.hs:138-149) calls it with n = occupied.
static long idx_dim2_to_flat(long dim, long x, long y) {
  auto calc = [&](long w) {
    if (w <= 0) return 0L;   // takeZero: [0] for w == 0, [] for w < 0
    long s = 0;
    for (long k = 0; k < w; ++k) s += dim - k;
    return s;
  };
  return x <= y ? calc(x) + (y - x) : calc(y) + (x - y);
}
static long sum_index_triang(long n) { return (n * n + n) / 2; }
static long sum_first_index(long n) {
  long s = n + sum_index_triang(n - 1);
  for (long k = 1; k <= n - 1; ++k) s += sum_index_triang(n) - k;
  return s;
}
static long four_index_to_flat(long n, long i, long j, long k, long l) {
  long a0 = 0;
  for (long m = 0; m < i; ++m) a0 += sum_first_index(n - m);
  long pos;
  if (i == j && j == k) {
    pos = l - i;
  } else if (i == j) {
    const long sh = i + 1;
    pos = (n - i) + idx_dim2_to_flat(n - sh, k - sh, l - sh);
  } else {
    pos = (n - i) + sum_index_triang(n - 1 - i);
    for (long m = 1; m <= j - 1 - i; ++m) pos += sum_index_triang(n - i) - m;
    pos += idx_dim2_to_flat(n, k, l) - idx_dim2_to_flat(n, i, j);
  }
  return a0 + pos;
}
static void sort_keys(long& i, long& j, long& k, long& l) {
  if (i > j) std::swap(i, j);
  if (k > l) std::swap(k, l);
  if (i > k || (i == k && j > l)) {
    std::swap(i, k);
    std::swap(j, l);
  }
}

__global__ void k_harris(long ntri, int nocc, const long* __restrict__ f1, const long* __restrict__ f2,
                         const double* __restrict__ eri, const double* __restrict__ H, double* __restrict__ out) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= ntri) return;
  double s = 0;
  for (int k = 0; k < nocc; ++k) s += eri[f1[idx * nocc + k]] - 0.5 * eri[f2[idx * nocc + k]];
  out[idx] = H[idx] + 2.0 * s;
}

static double nuclear_rep(const Basis& b) {
  // nuclearRep (HartreeFock.hs:300-305)
  double e = 0;
  for (int a = 0; a < b.natoms; ++a)
    for (int c = a + 1; c < b.natoms; ++c) {
      double r2 = 0;
      for (int x = 0; x < 3; ++x) r2 += (b.xyz[3 * a + x] - b.xyz[3 * c + x]) * (b.xyz[3 * a + x] - b.xyz[3 * c + x]);
      e += b.Z[a] * b.Z[c] / std::sqrt(r2);
    }
  return e;
}

namespace {
struct Hist {
  int slot_e, slot_f;
};
}

gbhf_status scf_run(gbhf_ctx* c, const gbhf_scf_opts* o, gbhf_result* r) {
  const Basis& b = c->basis;
  if (!c->basis_dev) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf: no basis set");
  if (b.nmol != 1) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf: the context holds a batch; call gbhf_set_basis");
  const int n = b.nbf;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  const bool ref = o->mode == GBHF_MODE_REFERENCE;
  if (o->diis_size < 1 || o->diis_size > 8) return fail(c, GBHF_ERR_BAD_INPUT, "diis_size must be 1..8");
  if (o->max_iter < 1) return fail(c, GBHF_ERR_BAD_INPUT, "max_iter must be >= 1");
  double zsum = 0;
  for (double z : b.Z) zsum += z;
  const int nocc = (int)std::floor((zsum - o->charge) / 2.0);
  if (nocc < 0 || nocc > n) return fail(c, GBHF_ERR_BAD_INPUT, "occupied orbitals out of range");
  const double enuc = nuclear_rep(b);
  GBHF_TRY(ensure_boys_tables(c));
  GBHF_WS(c, S, 0, nn);
  GBHF_WS(c, H, 1, nn);
  GBHF_WS(c, X, 2, nn);
  GBHF_WS(c, D, 3, nn);
  GBHF_WS(c, F, 4, nn);
  GBHF_WS(c, Gacc, 5, nn);
  GBHF_WS(c, Gpp, 6, nn);
  GBHF_WS(c, E, 7, nn);
  GBHF_WS(c, Cm, 8, nn);
  GBHF_WS(c, Fd, 9, nn);
  GBHF_WS(c, fS, 15, ntri);
  GBHF_WS(c, fH, 16, ntri);
  GBHF_WS(c, fD, 17, ntri);
  GBHF_WS(c, Cp, 18, nn);
  GBHF_WS(c, eps, 19, (size_t)n);
  GBHF_WS(c, Dnew, 20, nn);
  GBHF_WS(c, Dref, 21, nn);
  GBHF_WS(c, coefs, 22, 32);
  using clk = std::chrono::steady_clock;
  auto ms_since = [](clk::time_point t0) {
    return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
  };
  auto t_phase = clk::now();
  // one-electron matrices and orthogonaliser
  GBHF_TRY(onee_matrices(c, ref, fS, fH));
  GBHF_TRY(flat_to_square(c, n, fS, S));
  GBHF_TRY(flat_to_square(c, n, fH, H));
  // Reference mode: symmOrtho as the reference writes it (U s^-1/2 U^T by an
  // eigen-solve); exact mode: the same S^-1/2 by Newton-Schulz (GEMMs only).
  if (ref) {
    GBHF_TRY(symm_ortho_dev(c, n, S, X));
  } else {
    int ns_iters = 0;
    GBHF_TRY(inv_sqrt_dev(c, n, S, X, &ns_iters));
  }
  // Per-iteration density: reference mode diagonalises (diagonalHF); exact
  // mode takes the same projector by purification (trace-correcting) and diagonalises
  // once at the end for the orbitals.
  auto new_density = [&](const double* Fsq, double* Dout) -> gbhf_status {
    if (ref) return diagonal_hf_dev(c, n, Fsq, X, nocc, Cm, Dout, eps, Cp);
    return density_purified_dev(c, n, Fsq, X, nocc, Dout);
  };
  // stored ERIs for the reference path (and the Harris guess)
  DBuf<double> eri;
  const long long P = (long long)ntri;
  const long long neri = P * (P + 1) / 2;
  const bool need_eri = ref || o->guess == GBHF_GUESS_HARRIS;
  if (need_eri) {
    if (b.maxL > 2) return fail(c, GBHF_ERR_UNSUPPORTED, "stored ERIs support s, p and d functions");
    if (neri > (1ll << 31)) return fail(c, GBHF_ERR_UNSUPPORTED, "stored canonical ERIs too large for this basis");
    GBHF_CUDA(c, eri.alloc((size_t)neri));
    GBHF_TRY(eri_canonical_dev(c, ref, eri.p));
  }
  // initial density
  GBHF_CUDA(c, cudaMemsetAsync(Cp, 0, nn * sizeof(double), c->stream));
  {
    // identity warm start
    std::vector<double> I(nn, 0.0);
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
    GBHF_CUDA(c, cudaMemcpyAsync(Cp, I.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (o->guess == GBHF_GUESS_HARRIS) {
    std::vector<long> f1(ntri * (size_t)std::max(nocc, 1)), f2(f1.size());
    for (size_t idx = 0; idx < ntri; ++idx)
      for (int k = 0; k < nocc; ++k) {
        long i = 0, j = (long)idx, kk = k, l = k;
        sort_keys(i, j, kk, l);
        const long a = four_index_to_flat(nocc, i, j, kk, l);
        long i2 = 0, j2 = k, k2 = k, l2 = (long)idx;
        sort_keys(i2, j2, k2, l2);
        const long bidx = four_index_to_flat(nocc, i2, j2, k2, l2);
        if (a < 0 || a >= neri || bidx < 0 || bidx >= neri)
          return fail(c, GBHF_ERR_INDEX,
                      "Harris guess: the reference's ERI lookup (HartreeFock.hs:143-146) is out of bounds for this basis");
        f1[idx * nocc + k] = a;
        f2[idx * nocc + k] = bidx;
      }
    DBuf<long> d1, d2;
    GBHF_CUDA(c, d1.alloc(f1.size()));
    GBHF_CUDA(c, d2.alloc(f2.size()));
    GBHF_CUDA(c, cudaMemcpyAsync(d1.p, f1.data(), f1.size() * sizeof(long), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(d2.p, f2.data(), f2.size() * sizeof(long), cudaMemcpyHostToDevice, c->stream));
    k_harris<<<(unsigned)((ntri + 127) / 128), 128, 0, c->stream>>>((long)ntri, nocc, d1.p, d2.p, eri.p, fH, fD);
    count_launch(c);
    GBHF_TRY(flat_to_square(c, n, fD, Fd));
    GBHF_TRY(new_density(Fd, D));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  } else if (o->guess == GBHF_GUESS_SAD) {
    GBHF_TRY(sad_density(c, D));
  } else if (o->guess == GBHF_GUESS_DENSITY) {
    if (!c->guess_D.p || c->guess_gen != c->basis_gen)
      return fail(c, GBHF_ERR_BAD_INPUT, "GBHF_GUESS_DENSITY: no density set for this basis (gbhf_set_guess_density)");
    GBHF_TRY(flat_to_square(c, n, c->guess_D.p, D));
  } else {
    GBHF_TRY(new_density(H, D));
  }
  if (!ref) eri.release();
  if (o->autotune && !ref && !c->tuned[0]) {
    GBHF_TRY(autotune_dev(c, 0, D, o->precision, o->schwarz_cutoff,
                          o->precision == GBHF_PREC_FP64 ? 0.0 : o->mixed_cutoff, 2, nullptr));
  }
  // DIIS history buffers: slots in c->w beyond the driver's
  const int maxstore = std::max(o->diis_size - 1, 0);
  std::vector<DBuf<double>> hbuf(2 * (maxstore + 1));
  for (auto& hb : hbuf) GBHF_CUDA(c, hb.alloc(nn));
  std::vector<int> free_slots;
  for (int i = 0; i < maxstore + 1; ++i) free_slots.push_back(i);
  std::vector<int> stored;                         // newest first: index into pairs of hbuf
  std::vector<std::vector<double>> Bst;            // dots among stored (newest first)
  bool diis_on = false;
  double e_prev = 0, energy = 0;
  bool have_prev = false, converged = false;
  // final_fp64: after converging in mixed precision, continue with full FP64
  // builds until converged again.  Incremental builds carry a noise floor near
  // 1e-11 Eh (each screened-out contribution of a build is below the absolute
  // cutoff but new ones are dropped every step), so the final phase never uses them.
  bool fp64_final_phase = false;
  int precision = o->precision;
  int step = 0, since_full = 1 << 30;
  // GBHF_SCF_TRACE=1: one line per step on stderr (energy, changes, DIIS size)
  const char* tr_env = std::getenv("GBHF_SCF_TRACE");
  const bool trace = tr_env && tr_env[0] == '1';
  double fock_builds = 0;
  const double* last_fuse = F;
  double hstats[4];
  GBHF_TRY(flush_jk_stats(c));
  const double prim64_0 = c->prof.prim64, prim32_0 = c->prof.prim32, shq0 = c->prof.shellq, fnq0 = c->prof.fnq;
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->prof.ph_setup += ms_since(t_phase);
  c->scf_trace.clear();
  // the purification checks of the loop ride on its statistics reads
  // (a record left pending by an SCF that stopped on an error is dropped with it)
  struct DeferGuard {
    gbhf_ctx* c;
    ~DeferGuard() {
      c->purify_defer = false;
      c->purify_pending = false;
    }
  } defer_guard{c};
  c->purify_pending = false;
  c->purify_defer = true;
  for (step = 0; step < o->max_iter; ++step) {
    // phase boundaries as events on the stream (read after the step's last
    // host synchronisation, so that no phase waits for the GPU to drain)
    GBHF_CUDA(c, cudaEventRecord(c->evp[0], c->stream));
    // ---- Fock matrix of the current density
    if (ref) {
      GBHF_TRY(square_to_flat(c, n, D, fD));
      GBHF_TRY(fock_canonical_dev(c, fH, fD, eri.p, fS /*tmp flat F*/));
      GBHF_TRY(flat_to_square(c, n, fS, F));
      fock_builds += 1;
    } else {
      const bool full = !o->incremental || since_full >= (o->full_rebuild_every > 0 ? o->full_rebuild_every : (1 << 30)) ||
                        step == 0 || fp64_final_phase;
      GBHF_CUDA(c, cudaMemsetAsync(Gpp, 0, nn * sizeof(double), c->stream));
      if (full) {
        GBHF_TRY(jk_build(c, D, Gpp, precision, o->schwarz_cutoff, o->mixed_cutoff, 1.0));
        GBHF_TRY(add_sym(c, n, nullptr, Gpp, Gacc));
        since_full = 1;
      } else {
        GBHF_TRY(axpby(c, nn, 1.0, D, -1.0, Dref, Dnew));   // dD (Dnew as scratch)
        // per-pair weights from the local size of dD (tighter than its global
        // max; a zero dD leaves the task lists empty)
        GBHF_TRY(jk_build(c, Dnew, Gpp, precision, o->schwarz_cutoff, o->mixed_cutoff, 1.0, true));
        GBHF_TRY(add_sym(c, n, Gacc, Gpp, Gacc));
        ++since_full;
      }
      GBHF_CUDA(c, cudaMemcpyAsync(Dref, D, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      GBHF_TRY(axpby(c, nn, 1.0, H, 1.0, Gacc, F));
      fock_builds += 1;
    }
    GBHF_CUDA(c, cudaEventRecord(c->evp[1], c->stream));
    // ---- DIIS error and extrapolation (DIIS.hs:55-132)
    GBHF_TRY(diis_error_dev(c, n, F, S, D, X, E));
    double maxe = 0;
    const double* Fuse = F;
    // newdots[j] = tr(e e_j) for stored j (newest first), newdots.back() = tr(e e);
    // max |e| and the dots come back in one copy
    std::vector<double> newdots;
    {
      std::vector<const double*> mats;
      for (int s : stored) mats.push_back(hbuf[2 * s].p);
      mats.push_back(E);
      const int nd = (int)mats.size();
      GBHF_TRY(dot_matrices(c, (int)nn, nd, mats.data(), E, coefs));
      GBHF_TRY(max_abs_dev(c, nn, E, coefs + nd));
      newdots.resize(nd + 1);
      GBHF_CUDA(c, cudaMemcpyAsync(newdots.data(), coefs, (nd + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                                   c->stream));
      GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
      maxe = newdots[nd];
      newdots.pop_back();
    }
    auto drop_oldest = [&]() {
      free_slots.push_back(stored.back());
      stored.pop_back();
      Bst.pop_back();
      for (auto& row : Bst) row.pop_back();
      newdots.erase(newdots.end() - 2);
    };
    // updateDIIS (DIIS.hs:111-114): prepend (e, F), keep at most diis_size-1
    auto prepend = [&]() -> gbhf_status {
      if (maxstore == 0) return GBHF_OK;
      if ((int)stored.size() >= maxstore) drop_oldest();
      const int slot = free_slots.back();
      free_slots.pop_back();
      GBHF_CUDA(c, cudaMemcpyAsync(hbuf[2 * slot].p, E, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      GBHF_CUDA(c, cudaMemcpyAsync(hbuf[2 * slot + 1].p, F, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      std::vector<double> row;
      row.push_back(newdots.back());
      for (size_t j = 0; j < stored.size(); ++j) row.push_back(newdots[j]);
      for (size_t i = 0; i < Bst.size(); ++i) Bst[i].insert(Bst[i].begin(), newdots[i]);
      Bst.insert(Bst.begin(), row);
      stored.insert(stored.begin(), slot);
      return GBHF_OK;
    };
    if (!diis_on) {
      if (step > 0 && maxe < o->diis_start) {   // diisDriver OFF branch
        GBHF_TRY(prepend());
        diis_on = true;
      }
    } else {
      // diis (DIIS.hs:70-88): current + stored; drop the oldest stored pair on failure
      while (true) {
        const int k = 1 + (int)stored.size();
        const int m = k + 1;
        std::vector<double> Bm((size_t)m * m, 0.0), rhs(m, 0.0), x(m, 0.0);
        for (int i = 0; i < k; ++i)
          for (int j = 0; j < k; ++j) {
            double v;
            if (i == 0 && j == 0) v = newdots.back();
            else if (i == 0) v = newdots[j - 1];
            else if (j == 0) v = newdots[i - 1];
            else v = Bst[i - 1][j - 1];
            Bm[(size_t)i * m + j] = v;
          }
        for (int i = 0; i < k; ++i) {
          Bm[(size_t)i * m + k] = -1.0;
          Bm[(size_t)k * m + i] = -1.0;
        }
        rhs[k] = -1.0;
        bool ok = false;
        GBHF_TRY(gauss_elem_dev_call(c, m, Bm.data(), rhs.data(), x.data(), &ok));
        if (ok) {
          std::vector<const double*> mats;
          mats.push_back(F);
          for (int s : stored) mats.push_back(hbuf[2 * s + 1].p);
          GBHF_CUDA(c, cudaMemcpyAsync(coefs, x.data(), k * sizeof(double), cudaMemcpyHostToDevice, c->stream));
          GBHF_TRY(lincomb(c, (int)nn, k, mats.data(), coefs, Fd));
          Fuse = Fd;
          break;
        }
        if (stored.empty()) return fail(c, GBHF_ERR_SINGULAR, "DIIS system singular with no stored vectors left");
        drop_oldest();
      }
      GBHF_TRY(prepend());
    }
    GBHF_CUDA(c, cudaEventRecord(c->evp[2], c->stream));
    // ---- diagonalise the (extrapolated) Fock matrix
    GBHF_TRY(new_density(Fuse, Dnew));
    last_fuse = o->ref_stop_rule ? Fuse : F;
    GBHF_CUDA(c, cudaEventRecord(c->evp[3], c->stream));
    // ---- energies and convergence
    double rms = 0;
    if (o->ref_stop_rule) {
      GBHF_TRY(reduce_stats(c, n, nullptr, H, Fuse, Dnew, D, hstats));
      energy = hstats[1] + enuc;   // variationalE with F_DIIS and the new density
      rms = std::sqrt(hstats[2] / (double)nn);
      converged = step != 0 && maxe < o->conv_error;
    } else {
      GBHF_TRY(reduce_stats(c, n, nullptr, H, F, Dnew, D, hstats));
      energy = hstats[3] + enuc;   // E[D] with F = F(D)
      rms = std::sqrt(hstats[2] / (double)nn);
      // with final_fp64 the mixed phase hands over at 1e-9 Eh / 1e-7 (the FP64 full
      // builds that follow reach the requested thresholds in a few steps)
      const bool handover = o->final_fp64 && precision == GBHF_PREC_MIXED;
      const double ce = handover ? std::max(o->conv_energy, 1e-9) : o->conv_energy;
      const double cd = handover ? std::max(o->conv_density, 1e-7) : o->conv_density;
      converged = have_prev && std::fabs(energy - e_prev) < ce && rms < cd;
      if (trace)
        std::fprintf(stderr, "gbhf scf %3d  E %.12f  dE %+.3e  rms(dD) %.3e  max|e| %.3e  diis %d  %s%s\n", step,
                     energy, have_prev ? energy - e_prev : 0.0, rms, maxe, diis_on ? (int)stored.size() : 0,
                     precision == GBHF_PREC_FP64 ? "fp64" : "mixed", fp64_final_phase ? " final" : "");
    }
    GBHF_CUDA(c, cudaEventRecord(c->evp[4], c->stream));
    GBHF_CUDA(c, cudaEventSynchronize(c->evp[4]));
    float ph[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) GBHF_CUDA(c, cudaEventElapsedTime(&ph[i], c->evp[i], c->evp[i + 1]));
    c->prof.ph_fock += ph[0];
    c->prof.ph_diis += ph[1];
    c->prof.ph_diag += ph[2];
    c->prof.ph_other += ph[3];
    {
      const double rec[GBHF_SCF_TRACE_FIELDS] = {
          (double)step, energy, have_prev ? energy - e_prev : 0.0, rms, maxe, diis_on ? (double)stored.size() : 0.0,
          fp64_final_phase ? 2.0 : (precision == GBHF_PREC_MIXED ? 1.0 : 0.0), (double)(ph[0] + ph[1] + ph[2] + ph[3])};
      c->scf_trace.insert(c->scf_trace.end(), rec, rec + GBHF_SCF_TRACE_FIELDS);
    }
    e_prev = energy;
    have_prev = true;
    GBHF_CUDA(c, cudaMemcpyAsync(D, Dnew, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (converged) {
      if (!ref && o->final_fp64 && precision == GBHF_PREC_MIXED) {
        precision = GBHF_PREC_FP64;
        fp64_final_phase = true;
        converged = false;
        have_prev = false;
        continue;
      }
      break;
    }
  }
  c->purify_defer = false;
  GBHF_TRY(purify_flush(c));
  // keep the converged state for gbhf_gradient
  GBHF_CUDA(c, c->last_D.alloc(nn));
  GBHF_CUDA(c, c->last_F.alloc(nn));
  GBHF_CUDA(c, cudaMemcpyAsync(c->last_D.p, D, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  GBHF_CUDA(c, cudaMemcpyAsync(c->last_F.p, last_fuse, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  c->last_nocc = nocc;
  c->last_gen = c->basis_gen;
  if (r && !ref && (r->coeff || r->orb_energies)) {
    // orbitals of the last diagonalised Fock matrix (one eigen-solve per SCF)
    GBHF_TRY(diagonal_hf_dev(c, n, last_fuse, X, nocc, Cm, Dnew, eps, Cp));
  }
  if (r) {
    GBHF_TRY(flush_jk_stats(c));
    r->energy = energy;
    r->iterations = std::min(step + 1, o->max_iter);
    r->converged = converged ? 1 : 0;
    r->n_occupied = nocc;
    r->nuclear_repulsion = enuc;
    r->fock_builds = fock_builds;
    r->eri_prim_quartets = (c->prof.prim64 - prim64_0) + (c->prof.prim32 - prim32_0);
    r->eri_fp32_fraction = r->eri_prim_quartets > 0 ? (c->prof.prim32 - prim32_0) / r->eri_prim_quartets : 0.0;
    r->eri_quartets = c->prof.shellq - shq0;
    r->eri_fn_quartets = c->prof.fnq - fnq0;
    // outputs: Fock (reference: F_DIIS), coefficients, new density, orbital energies
    if (r->fock_flat) {
      GBHF_TRY(square_to_flat(c, n, last_fuse, fS));
      GBHF_CUDA(c, cudaMemcpyAsync(r->fock_flat, fS, ntri * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    if (r->coeff) GBHF_CUDA(c, cudaMemcpyAsync(r->coeff, Cm, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (r->density_flat) {
      GBHF_TRY(square_to_flat(c, n, D, fD));
      GBHF_CUDA(c, cudaMemcpyAsync(r->density_flat, fD, ntri * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    if (r->orb_energies)
      GBHF_CUDA(c, cudaMemcpyAsync(r->orb_energies, eps, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (!converged) return fail(c, GBHF_ERR_NOT_CONVERGED, "SCF maxium steps exceeded");
  return GBHF_OK;
}

}  // namespace gbhf
