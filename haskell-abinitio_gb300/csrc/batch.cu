// gbhf_scf_batch: many independent molecules in one call (no counterpart in
// the reference, whose scfHF takes one molecule).
//
// The molecules become one basis with a molecule partition (atoms and
// functions contiguous per molecule), and the batched driver (bscf.cu) runs
// their SCFs together: one set of launches per step for all molecules, no
// shell pair or quartet across two molecules.
#include <string>
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
  const int n_atoms = atom_off[n_mol], n_cgf = cgf_off[n_mol];
  GBHF_TRY(build_basis_mols(c, n_atoms, xyz_bohr, charges, n_cgf, cgf_atom, cgf_lxyz, cgf_nprim, prim_coef, prim_exp,
                            n_mol, atom_off, cgf_off));
  return bscf_run(c, opts, energies, iterations, converged, grads);
}
