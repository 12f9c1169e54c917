// Device helpers shared by the dense kernels (single molecule and batched).
#pragma once
#include <cuda_runtime.h>

namespace gbhf {

// One m8n8k4 FP64 tensor-core product (DMMA): {d0, d1} += a * b for this lane's
// fragments (row-major A, column-major B).
static __device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

// Sum (or max) of v over the block; the result is valid in warp 0.
static __device__ __forceinline__ double block_reduce(double v, bool is_max) {
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, w) : v + w;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) / 32;
  v = threadIdx.x < nw ? sh[threadIdx.x] : (is_max ? 0.0 : 0.0);
  if (wid == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double w = __shfl_xor_sync(0xffffffffu, v, o);
      v = is_max ? fmax(v, w) : v + w;
    }
  }
  return v;
}

// gaussElem (NumericalTools/GaussElimination.hs:42-98), single thread: unpivoted
// elimination over all pivots, failure when a row of the eliminated matrix has
// no |entry| > 1e-6 or any entry is NaN/Inf, then back substitution.
static __device__ bool gauss_elem_dev(int m, double* a, double* b, double* x) {
  for (int k = 0; k < m; ++k) {
    const double piv = a[k * m + k];
    for (int i = k + 1; i < m; ++i) {
      const double alpha = a[i * m + k] / piv;
      for (int j = m - 1; j >= k; --j) a[i * m + j] = a[i * m + j] - alpha * a[k * m + j];
      b[i] = b[i] - alpha * b[k];
    }
  }
  for (int i = 0; i < m; ++i) {
    bool any = false;
    for (int j = 0; j < m; ++j) {
      const double v = a[i * m + j];
      if (isnan(v) || isinf(v)) return false;
      if (fabs(v) > 1e-6) any = true;
    }
    if (!any) return false;
  }
  for (int k = m - 1; k >= 0; --k) {
    double s = 0;
    for (int j = k + 1; j < m; ++j) s += x[j] * a[k * m + j];
    x[k] = (b[k] - s) * (1.0 / a[k * m + k]);
  }
  return true;
}

}  // namespace gbhf
