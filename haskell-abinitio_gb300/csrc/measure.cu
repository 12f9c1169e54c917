// Measurement entry points: stream events, L2 flush, CUDA-core FMA peaks,
// per-class J/K statistics.
#include <algorithm>

#include "gbhf_internal.h"

using namespace gbhf;

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T seed, T* out) {
  // 8 independent FMA chains per thread keep the pipe busy; the result is
  // stored so the compiler cannot drop the work.
  T a0 = seed + threadIdx.x, a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
  T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
  const T m = T(0.999999), c = T(1e-7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
      a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
    }
  }
  const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == T(-1)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

gbhf_status gbhf_profile_classes(gbhf_ctx* c, double* out) {
  if (!c || !out) return GBHF_ERR_BAD_INPUT;
  GBHF_TRY(gbhf::flush_jk_stats(c));
  for (int k = 0; k < gbhf::NCOMBO; ++k)
    for (int p = 0; p < 2; ++p)
      for (int q = 0; q < 4; ++q) out[(k * 2 + p) * 4 + q] = c->prof.cls[k][p][q];
  return GBHF_OK;
}

gbhf_status gbhf_event_record(gbhf_ctx* c, int slot) {
  if (!c || slot < 0 || slot >= 8) return GBHF_ERR_BAD_INPUT;
  GBHF_CUDA(c, cudaSetDevice(c->device));
  GBHF_CUDA(c, cudaEventRecord(c->evu[slot], c->stream));
  return GBHF_OK;
}

gbhf_status gbhf_event_elapsed(gbhf_ctx* c, int a, int b, double* ms) {
  if (!c || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return GBHF_ERR_BAD_INPUT;
  GBHF_CUDA(c, cudaEventSynchronize(c->evu[b]));
  float f = 0;
  GBHF_CUDA(c, cudaEventElapsedTime(&f, c->evu[a], c->evu[b]));
  *ms = f;
  return GBHF_OK;
}

gbhf_status gbhf_flush_l2(gbhf_ctx* c) {
  if (!c) return GBHF_ERR_BAD_INPUT;
  GBHF_CUDA(c, cudaSetDevice(c->device));
  const size_t bytes = 256u << 20;
  GBHF_CUDA(c, c->flush.alloc(bytes));
  GBHF_CUDA(c, cudaMemsetAsync(c->flush.p, (int)(c->prof.launches & 0xff), bytes, c->stream));
  return GBHF_OK;
}

gbhf_status gbhf_peak_flops(gbhf_ctx* c, int precision, double* tflops) {
  if (!c || !tflops) return GBHF_ERR_BAD_INPUT;
  GBHF_CUDA(c, cudaSetDevice(c->device));
  const int blocks = c->nsm * 8, threads = 256;
  DBuf<double> out;
  GBHF_CUDA(c, out.alloc((size_t)blocks * threads));
  cudaEvent_t e0, e1;
  GBHF_CUDA(c, cudaEventCreate(&e0));
  GBHF_CUDA(c, cudaEventCreate(&e1));
  const bool fp64 = precision == GBHF_PREC_FP64;
  const int iters = fp64 ? 256 : 8192;
  // warm-up, then timed run
  for (int rep = 0; rep < 2; ++rep) {
    if (rep == 1) GBHF_CUDA(c, cudaEventRecord(e0, c->stream));
    if (fp64)
      k_fma_peak<double><<<blocks, threads, 0, c->stream>>>(iters, 1.0, out.p);
    else
      k_fma_peak<float><<<blocks, threads, 0, c->stream>>>(iters, 1.0f, (float*)out.p);
    count_launch(c);
  }
  GBHF_CUDA(c, cudaEventRecord(e1, c->stream));
  GBHF_CUDA(c, cudaEventSynchronize(e1));
  float ms = 0;
  GBHF_CUDA(c, cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double fmas = (double)blocks * threads * iters * 16.0 * 8.0;
  *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  return GBHF_OK;
}

}  // extern "C"
