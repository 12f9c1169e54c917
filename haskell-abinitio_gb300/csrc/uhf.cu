// Open-shell (unrestricted) Hartree-Fock: the multiplicity the reference's
// command line accepts and then ignores (--multi, Main.hs:55, OptsCheck.hs:31).
//
// n_alpha - n_beta = multiplicity - 1.  With D_T = D_a + D_b and the spin
// density D_s = D_a - D_b (D_sigma = C_sigma,occ C_sigma,occ^T),
//   F_a = H + J(D_T) - K(D_a) = H + G(D_T) - K(D_s)/2,
//   F_b = H + J(D_T) - K(D_b) = H + G(D_T) + K(D_s)/2,
// with G(D) = J(D) - K(D)/2 the closed-shell build of the J/K kernels and the
// exchange-only build for K(D_s).  E = 1/2 [tr(D_T H) + tr(D_a F_a) + tr(D_b F_b)]
// + V_nn.  DIIS extrapolates F_a and F_b with one set of coefficients from the
// summed error products; each spin's density comes from the eigenvectors of
// its Fock matrix (Jacobi, warm-started from the previous step's vectors):
// open shells often have a degenerate highest occupied level in one spin
// (OH: one electron in the pi pair), where purification has no gap to work
// with and the eigen-solve picks one orbital of the pair.  Full builds every step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "gbhf_internal.h"

namespace gbhf {

static double nuclear_rep_u(const Basis& b) {
  double e = 0;
  for (int a = 0; a < b.natoms; ++a)
    for (int c = a + 1; c < b.natoms; ++c) {
      double r2 = 0;
      for (int x = 0; x < 3; ++x) r2 += (b.xyz[3 * a + x] - b.xyz[3 * c + x]) * (b.xyz[3 * a + x] - b.xyz[3 * c + x]);
      e += b.Z[a] * b.Z[c] / std::sqrt(r2);
    }
  return e;
}

// Solve the bordered DIIS system (k vectors) by Gaussian elimination with
// partial pivoting; false when singular.
static bool diis_solve(int k, const std::vector<double>& B, std::vector<double>& x) {
  const int m = k + 1;
  std::vector<double> a((size_t)m * (m + 1), 0.0);
  for (int i = 0; i < k; ++i) {
    for (int j = 0; j < k; ++j) a[(size_t)i * (m + 1) + j] = B[(size_t)i * k + j];
    a[(size_t)i * (m + 1) + k] = -1.0;
    a[(size_t)k * (m + 1) + i] = -1.0;
  }
  a[(size_t)k * (m + 1) + m] = -1.0;
  for (int col = 0; col < m; ++col) {
    int piv = col;
    for (int r = col + 1; r < m; ++r)
      if (std::fabs(a[(size_t)r * (m + 1) + col]) > std::fabs(a[(size_t)piv * (m + 1) + col])) piv = r;
    if (!(std::fabs(a[(size_t)piv * (m + 1) + col]) > 1e-300)) return false;
    if (piv != col)
      for (int j = 0; j <= m; ++j) std::swap(a[(size_t)piv * (m + 1) + j], a[(size_t)col * (m + 1) + j]);
    for (int r = 0; r < m; ++r) {
      if (r == col) continue;
      const double f = a[(size_t)r * (m + 1) + col] / a[(size_t)col * (m + 1) + col];
      for (int j = col; j <= m; ++j) a[(size_t)r * (m + 1) + j] -= f * a[(size_t)col * (m + 1) + j];
    }
  }
  x.assign(k, 0.0);
  for (int i = 0; i < k; ++i) x[i] = a[(size_t)i * (m + 1) + m] / a[(size_t)i * (m + 1) + i];
  return true;
}

gbhf_status uhf_run(gbhf_ctx* c, const gbhf_scf_opts* o, int multiplicity, gbhf_uhf_result* r) {
  const Basis& b = c->basis;
  if (!c->basis_dev) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_uhf: no basis set");
  if (b.nmol != 1) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_uhf: the context holds a batch");
  if (o->mode != GBHF_MODE_EXACT) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_uhf: exact mode (direct J/K) only");
  if (o->diis_size < 1 || o->diis_size > 8) return fail(c, GBHF_ERR_BAD_INPUT, "diis_size must be 1..8");
  if (o->max_iter < 1) return fail(c, GBHF_ERR_BAD_INPUT, "max_iter must be >= 1");
  if (o->guess != GBHF_GUESS_CORE && o->guess != GBHF_GUESS_SAD)
    return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_uhf: core or SAD guess");
  const int n = b.nbf;
  const size_t nn = (size_t)n * n, ntri = (size_t)n * (n + 1) / 2;
  double zsum = 0;
  for (double z : b.Z) zsum += z;
  const double nel_d = zsum - o->charge;
  const long nel = std::lround(nel_d);
  if (std::fabs(nel_d - (double)nel) > 1e-9 || nel < 0)
    return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_uhf: non-integer or negative electron count");
  if (multiplicity < 1 || (nel + multiplicity - 1) % 2 != 0 || multiplicity - 1 > nel)
    return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_uhf: multiplicity incompatible with the electron count");
  const int na = (int)((nel + multiplicity - 1) / 2), nb = (int)(nel - na);
  if (na > n) return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_uhf: more alpha electrons than basis functions");
  const double enuc = nuclear_rep_u(b);
  GBHF_TRY(ensure_boys_tables(c));
  DBuf<double> S, H, X, Da, Db, DT, Ds, Fa, Fb, GT, GK, Gpp, Ea, Eb, Fxa, Fxb, Na, Nb, T1, fS, fH, fT, eps, Cm, Cpa,
      Cpb, dots;
  for (DBuf<double>* m : {&S, &H, &X, &Da, &Db, &DT, &Ds, &Fa, &Fb, &GT, &GK, &Gpp, &Ea, &Eb, &Fxa, &Fxb, &Na, &Nb,
                          &T1, &Cm, &Cpa, &Cpb})
    GBHF_CUDA(c, m->alloc(nn));
  {   // identity warm starts of the two eigen-solves
    std::vector<double> I(nn, 0.0);
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
    GBHF_CUDA(c, cudaMemcpyAsync(Cpa.p, I.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(Cpb.p, I.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  GBHF_CUDA(c, fS.alloc(ntri));
  GBHF_CUDA(c, fH.alloc(ntri));
  GBHF_CUDA(c, fT.alloc(ntri));
  GBHF_CUDA(c, eps.alloc(n));
  GBHF_CUDA(c, dots.alloc(256));   // [0, 224): dot products, [224, 256): DIIS coefficients
  GBHF_TRY(onee_matrices(c, false, fS.p, fH.p));
  GBHF_TRY(flat_to_square(c, n, fS.p, S.p));
  GBHF_TRY(flat_to_square(c, n, fH.p, H.p));
  int ns_iters = 0;
  GBHF_TRY(inv_sqrt_dev(c, n, S.p, X.p, &ns_iters));
  // density of one spin: C_occ C_occ^T (the closed-shell routine returns twice that)
  auto spin_density = [&](const double* F, int nocc, double* D, double* Cwarm) -> gbhf_status {
    GBHF_TRY(diagonal_hf_dev(c, n, F, X.p, nocc, Cm.p, T1.p, eps.p, Cwarm));
    return axpby(c, nn, 0.5, T1.p, 0.0, T1.p, D);
  };
  if (o->guess == GBHF_GUESS_SAD) {   // spin-unpolarised atoms: D_a = D_b = D_SAD / 2
    GBHF_TRY(sad_density(c, T1.p));
    GBHF_TRY(axpby(c, nn, 0.5, T1.p, 0.0, T1.p, Da.p));
    GBHF_CUDA(c, cudaMemcpyAsync(Db.p, Da.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  } else {
    GBHF_TRY(spin_density(H.p, na, Da.p, Cpa.p));
    GBHF_TRY(spin_density(H.p, nb, Db.p, Cpb.p));
  }
  // host scalars from device dot products
  auto dotv = [&](std::vector<std::pair<const double*, const double*>> prs, std::vector<double>& out) -> gbhf_status {
    out.resize(prs.size());
    for (size_t i = 0; i < prs.size(); ++i) {
      const double* mats[1] = {prs[i].first};
      GBHF_TRY(dot_matrices(c, (int)nn, 1, mats, prs[i].second, dots.p + i));
    }
    GBHF_CUDA(c, cudaMemcpyAsync(out.data(), dots.p, prs.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
    return GBHF_OK;
  };
  // DIIS history (current + up to diis_size - 1 stored), newest first
  const int maxstore = std::max(o->diis_size - 1, 0);
  std::vector<DBuf<double>> hist(4 * (maxstore + 1));
  for (auto& h : hist) GBHF_CUDA(c, h.alloc(nn));
  std::vector<int> stored, free_slots;
  for (int i = maxstore; i >= 0; --i) free_slots.push_back(i);
  auto slot = [&](int s, int which) { return hist[4 * s + which].p; };   // 0 e_a, 1 e_b, 2 F_a, 3 F_b
  double energy = 0, e_prev = 0;
  bool have_prev = false, converged = false;
  int step = 0;
  c->scf_trace.clear();
  for (step = 0; step < o->max_iter; ++step) {
    const auto t_step = std::chrono::steady_clock::now();
    GBHF_TRY(axpby(c, nn, 1.0, Da.p, 1.0, Db.p, DT.p));
    GBHF_TRY(axpby(c, nn, 1.0, Da.p, -1.0, Db.p, Ds.p));
    GBHF_CUDA(c, cudaMemsetAsync(Gpp.p, 0, nn * sizeof(double), c->stream));
    GBHF_TRY(jk_build(c, DT.p, Gpp.p, o->precision, o->schwarz_cutoff, o->mixed_cutoff, 1.0));
    GBHF_TRY(add_sym(c, n, nullptr, Gpp.p, GT.p));
    GBHF_CUDA(c, cudaMemsetAsync(Gpp.p, 0, nn * sizeof(double), c->stream));
    GBHF_TRY(jk_build(c, Ds.p, Gpp.p, o->precision, o->schwarz_cutoff, o->mixed_cutoff, 1.0, false, false));
    GBHF_TRY(add_sym(c, n, nullptr, Gpp.p, GK.p));   // -K(D_s)/2
    GBHF_TRY(axpby(c, nn, 1.0, H.p, 1.0, GT.p, T1.p));
    GBHF_TRY(axpby(c, nn, 1.0, T1.p, 1.0, GK.p, Fa.p));
    GBHF_TRY(axpby(c, nn, 1.0, T1.p, -1.0, GK.p, Fb.p));
    std::vector<double> tr;
    GBHF_TRY(dotv({{DT.p, H.p}, {Da.p, Fa.p}, {Db.p, Fb.p}}, tr));
    energy = 0.5 * (tr[0] + tr[1] + tr[2]) + enuc;
    // DIIS errors of both spins
    GBHF_TRY(diis_error_dev(c, n, Fa.p, S.p, Da.p, X.p, Ea.p));
    GBHF_TRY(diis_error_dev(c, n, Fb.p, S.p, Db.p, X.p, Eb.p));
    double ma = 0, mb = 0;
    GBHF_TRY(max_abs(c, nn, Ea.p, &ma));
    GBHF_TRY(max_abs(c, nn, Eb.p, &mb));
    const double maxe = std::max(ma, mb);
    // store the current pair (at most diis_size pairs), dropping the oldest
    {
      if ((int)stored.size() == maxstore + 1) {
        free_slots.push_back(stored.back());
        stored.pop_back();
      }
      const int sl = free_slots.back();
      free_slots.pop_back();
      GBHF_CUDA(c, cudaMemcpyAsync(slot(sl, 0), Ea.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      GBHF_CUDA(c, cudaMemcpyAsync(slot(sl, 1), Eb.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      GBHF_CUDA(c, cudaMemcpyAsync(slot(sl, 2), Fa.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      GBHF_CUDA(c, cudaMemcpyAsync(slot(sl, 3), Fb.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      stored.insert(stored.begin(), sl);
    }
    const double* Fua = Fa.p;
    const double* Fub = Fb.p;
    while (step > 0 && stored.size() >= 2 && maxe < o->diis_start) {
      const int k = (int)stored.size();
      std::vector<std::pair<const double*, const double*>> prs;
      for (int i = 0; i < k; ++i)
        for (int j = i; j < k; ++j) {
          prs.push_back({slot(stored[i], 0), slot(stored[j], 0)});
          prs.push_back({slot(stored[i], 1), slot(stored[j], 1)});
        }
      std::vector<double> v;
      GBHF_TRY(dotv(prs, v));
      std::vector<double> B((size_t)k * k);
      size_t q = 0;
      for (int i = 0; i < k; ++i)
        for (int j = i; j < k; ++j, q += 2) B[(size_t)i * k + j] = B[(size_t)j * k + i] = v[q] + v[q + 1];
      std::vector<double> x;
      if (diis_solve(k, B, x)) {
        std::vector<const double*> ma_, mb_;
        for (int i = 0; i < k; ++i) {
          ma_.push_back(slot(stored[i], 2));
          mb_.push_back(slot(stored[i], 3));
        }
        GBHF_CUDA(c, cudaMemcpyAsync(dots.p + 224, x.data(), k * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        GBHF_TRY(lincomb(c, (int)nn, k, ma_.data(), dots.p + 224, Fxa.p));
        GBHF_TRY(lincomb(c, (int)nn, k, mb_.data(), dots.p + 224, Fxb.p));
        Fua = Fxa.p;
        Fub = Fxb.p;
        break;
      }
      free_slots.push_back(stored.back());   // singular: drop the oldest and retry
      stored.pop_back();
    }
    GBHF_TRY(spin_density(Fua, na, Na.p, Cpa.p));
    GBHF_TRY(spin_density(Fub, nb, Nb.p, Cpb.p));
    GBHF_TRY(axpby(c, nn, 1.0, Na.p, -1.0, Da.p, T1.p));
    GBHF_TRY(axpby(c, nn, 1.0, Nb.p, -1.0, Db.p, Ds.p));
    std::vector<double> dd;
    GBHF_TRY(dotv({{T1.p, T1.p}, {Ds.p, Ds.p}}, dd));
    const double rms = std::sqrt((dd[0] + dd[1]) / (2.0 * (double)nn));
    converged = have_prev && std::fabs(energy - e_prev) < o->conv_energy && rms < o->conv_density;
    {
      const double rec[GBHF_SCF_TRACE_FIELDS] = {
          (double)step, energy, have_prev ? energy - e_prev : 0.0, rms, maxe, (double)stored.size(),
          o->precision == GBHF_PREC_MIXED ? 1.0 : 0.0,
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_step).count()};
      c->scf_trace.insert(c->scf_trace.end(), rec, rec + GBHF_SCF_TRACE_FIELDS);
    }
    e_prev = energy;
    have_prev = true;
    GBHF_CUDA(c, cudaMemcpyAsync(Da.p, Na.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(Db.p, Nb.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (converged) break;
  }
  if (converged) {
    // keep the converged state for gbhf_gradient_uhf: D_a, D_b and
    // W = D_a F_a D_a + D_b F_b D_b (= sum_s C_s,occ eps_s C_s,occ^T)
    GBHF_CUDA(c, c->last_uDa.alloc(nn));
    GBHF_CUDA(c, c->last_uDb.alloc(nn));
    GBHF_CUDA(c, c->last_uW.alloc(nn));
    GBHF_CUDA(c, cudaMemcpyAsync(c->last_uDa.p, Da.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    GBHF_CUDA(c, cudaMemcpyAsync(c->last_uDb.p, Db.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, Fa.p, n, Da.p, n, 0.0, T1.p, n));
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, Da.p, n, T1.p, n, 0.0, c->last_uW.p, n, true));
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, Fb.p, n, Db.p, n, 0.0, T1.p, n));
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, Db.p, n, T1.p, n, 1.0, c->last_uW.p, n, true));
    c->last_ugen = c->basis_gen;
  }
  if (r) {
    r->energy = energy;
    r->iterations = std::min(step + 1, o->max_iter);
    r->converged = converged ? 1 : 0;
    r->n_alpha = na;
    r->n_beta = nb;
    // <S^2> = Sz (Sz + 1) + n_b - tr(D_a S D_b S)
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, Da.p, n, S.p, n, 0.0, T1.p, n));
    GBHF_TRY(gemm(c, false, false, n, n, n, 1.0, S.p, n, T1.p, n, 0.0, Ds.p, n));
    std::vector<double> ov;
    GBHF_TRY(dotv({{Ds.p, Db.p}}, ov));
    const double sz = 0.5 * (na - nb);
    r->s2 = sz * (sz + 1) + nb - ov[0];
    for (int sp = 0; sp < 2; ++sp) {
      double* dflat = sp == 0 ? r->density_alpha_flat : r->density_beta_flat;
      double* oe = sp == 0 ? r->orb_energies_alpha : r->orb_energies_beta;
      const double* Dsp = sp == 0 ? Da.p : Db.p;
      if (dflat) {
        GBHF_TRY(square_to_flat(c, n, Dsp, fT.p));
        GBHF_CUDA(c, cudaMemcpyAsync(dflat, fT.p, ntri * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
      }
      if (oe) {
        GBHF_TRY(diagonal_hf_dev(c, n, sp == 0 ? Fa.p : Fb.p, X.p, sp == 0 ? na : nb, Cm.p, T1.p, eps.p,
                                 sp == 0 ? Cpa.p : Cpb.p));
        GBHF_CUDA(c, cudaMemcpyAsync(oe, eps.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
      }
    }
  }
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  if (!converged) return fail(c, GBHF_ERR_NOT_CONVERGED, "UHF: maximum steps exceeded");
  return GBHF_OK;
}

}  // namespace gbhf
