// gbhf_scf_batch: many independent molecules in one call.
//
// Small molecules leave most of the GPU idle (a (H2O)_3 STO-3G Fock build is a
// few thousand quartets), so the batch keeps several SCFs in flight at once:
// a pool of worker contexts, each with its own CUDA stream and host thread,
// takes molecules largest-first from a shared counter.  Their kernels overlap
// on the device; there is no data exchange between molecules.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "gbhf_internal.h"

extern "C" gbhf_status gbhf_scf_batch(gbhf_ctx* c, int n_mol, const int* atom_off, const int* cgf_off,
                                      const double* xyz_bohr, const double* charges, const int* cgf_atom,
                                      const int* cgf_lxyz, const int* cgf_nprim, const double* prim_coef,
                                      const double* prim_exp, const gbhf_scf_opts* opts, double* energies,
                                      int* iterations, int* converged, double* grads) {
  using namespace gbhf;
  if (!c) return GBHF_ERR_BAD_INPUT;
  PoolScope pool_scope(c);
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, GBHF_ERR_CUDA, "cudaSetDevice");
  c->err.clear();
  if (n_mol < 0 || (n_mol > 0 && (!atom_off || !cgf_off || !xyz_bohr || !charges || !cgf_atom || !cgf_lxyz ||
                                  !cgf_nprim || !prim_coef || !prim_exp || !opts || !energies)))
    return fail(c, GBHF_ERR_BAD_INPUT, "gbhf_scf_batch: bad arguments");
  if (n_mol == 0) return GBHF_OK;
  // primitive offsets of each CGF in the concatenated arrays
  const int total_cgf = cgf_off[n_mol];
  std::vector<long> prim_off(total_cgf + 1, 0);
  for (int k = 0; k < total_cgf; ++k) prim_off[k + 1] = prim_off[k] + cgf_nprim[k];
  // largest first (cost ~ n^4)
  std::vector<int> order(n_mol);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (cgf_off[a + 1] - cgf_off[a]) > (cgf_off[b + 1] - cgf_off[b]);
  });
  const int nworkers = std::max(1, std::min(n_mol, 16));
  // worker contexts are kept in the parent context between calls
  static std::mutex pool_mutex;
  {
    std::lock_guard<std::mutex> lock(pool_mutex);
    while ((int)c->pool.size() < nworkers) {
      gbhf_ctx* w = nullptr;
      gbhf_status s = gbhf_create(&w, c->device);
      if (s != GBHF_OK) return fail(c, s, "gbhf_scf_batch: cannot create a worker context");
      c->pool.push_back(w);
    }
  }
  std::atomic<int> next(0);
  std::vector<gbhf_status> status(n_mol, GBHF_OK);
  std::vector<std::string> msgs(n_mol);
  auto work = [&](int wi) {
    gbhf_ctx* w = c->pool[wi];
    cudaSetDevice(w->device);
    while (true) {
      const int slot = next.fetch_add(1);
      if (slot >= n_mol) break;
      const int m = order[slot];
      const int a0 = atom_off[m], a1 = atom_off[m + 1], f0 = cgf_off[m], f1 = cgf_off[m + 1];
      const int na = a1 - a0, nf = f1 - f0;
      std::vector<int> atom_local(nf);
      for (int k = 0; k < nf; ++k) atom_local[k] = cgf_atom[f0 + k] - a0;
      gbhf_status s = gbhf_set_basis(w, na, xyz_bohr + 3 * a0, charges + a0, nf, atom_local.data(),
                                     cgf_lxyz + 3 * f0, cgf_nprim + f0, prim_coef + prim_off[f0],
                                     prim_exp + prim_off[f0]);
      gbhf_result r{};
      if (s == GBHF_OK) s = gbhf_scf(w, opts, &r);
      energies[m] = r.energy;
      if (iterations) iterations[m] = r.iterations;
      if (converged) converged[m] = r.converged;
      if (s == GBHF_OK && grads) s = gbhf_gradient(w, opts->precision, opts->schwarz_cutoff > 0 ? opts->schwarz_cutoff : 1e-12,
                                                   nullptr, nullptr, grads + 3 * a0);
      status[m] = s;
      if (s != GBHF_OK) msgs[m] = w->err;
    }
  };
  std::vector<std::thread> threads;
  for (int wi = 1; wi < nworkers; ++wi) threads.emplace_back(work, wi);
  work(0);
  for (auto& t : threads) t.join();
  // aggregate statistics into the parent context
  for (int wi = 0; wi < nworkers; ++wi) {
    const Profile& p = c->pool[wi]->prof;
    c->prof.prim64 += p.prim64;
    c->prof.prim32 += p.prim32;
    c->prof.shellq += p.shellq;
    c->prof.fnq += p.fnq;
    c->prof.launches += p.launches;
    c->pool[wi]->prof = Profile();
  }
  for (int m = 0; m < n_mol; ++m)
    if (status[m] != GBHF_OK) return fail(c, status[m], "molecule " + std::to_string(m) + ": " + msgs[m]);
  return GBHF_OK;
}
