// Parallel cyclic Jacobi eigen-solver kernels (defined in linalg.cu).
#pragma once
#include <cuda_runtime.h>

namespace gbhf {

struct JacobiArgs {
  int n, m;            // matrix size, padded even size
  double* A;           // m x m (padded with zeros), destroyed; holds the diagonalised matrix on return
  double* A2;          // m x m second buffer (rounds alternate between A and A2)
  double* V;           // n x m accumulated rotations (rows n)
  double* rot;         // two rounds' rotations: per index alpha, beta (2 x 2m)
  double* red;         // reduction scratch (2 doubles)
  unsigned* bar;       // barrier count, generation (must start at 0)
  int* status;         // device status word (must start at 0)
  int max_sweeps;
  double tol;          // relative off-diagonal Frobenius tolerance
  int* sweeps_out;
};

// One cooperative launch (all blocks co-resident), 256 threads per block.
__global__ void __launch_bounds__(256) k_jacobi(JacobiArgs a);
// A <- Ain padded to m x m, V <- identity (n x m).
__global__ void k_jacobi_init(int n, int m, const double* __restrict__ Ain, double* __restrict__ A,
                              double* __restrict__ V);
// Ascending sort of diag(A) with the matching columns of V; one block of 1024 threads, n <= 1024.
__global__ void k_sort_eig(int n, int m, const double* __restrict__ A, const double* __restrict__ V,
                           double* __restrict__ evals, double* __restrict__ evecs);

}  // namespace gbhf
