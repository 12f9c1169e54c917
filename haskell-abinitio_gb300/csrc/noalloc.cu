// Eigen-solve entry point that allocates nothing.
//
// Some callers cannot allocate device memory while they call us: code that
// runs inside another framework's custom-call or plugin hook, where the host
// framework owns every device buffer and its memory planner forbids
// cudaMalloc.  They hand in device buffers for the input matrix and the
// results and nothing else.  This entry point serves them: the Jacobi
// solver's working memory lives in the file-scope array g_eigen_scratch
// below, sized for matrices up to GBHF_NOALLOC_EIGEN_MAX_N, which every GPU
// that loads the library keeps for the life of the process.  Every call waits
// for the caller's stream to finish before it returns (it reads back the
// solver's status word).
#include <mutex>

#include "gbhf_internal.h"
#include "jacobi.cuh"

namespace {

constexpr int kMaxN = GBHF_NOALLOC_EIGEN_MAX_N;
// Layout (doubles): A (kMaxN^2) | A2 (kMaxN^2, the second Jacobi buffer) | V (kMaxN^2) |
// rot (4 kMaxN) | red (4) | ints (8 doubles' worth: barrier count and generation, status, sweeps)
constexpr size_t kOffA = 0;
constexpr size_t kOffA2 = kOffA + (size_t)kMaxN * kMaxN;
constexpr size_t kOffV = kOffA2 + (size_t)kMaxN * kMaxN;
constexpr size_t kOffRot = kOffV + (size_t)kMaxN * kMaxN;
constexpr size_t kOffRed = kOffRot + 4 * (size_t)kMaxN;
constexpr size_t kOffInts = kOffRed + 4;
constexpr size_t kScratchDoubles = kOffInts + 8;   // barrier, status, sweeps

static __device__ __align__(256) double g_eigen_scratch[kScratchDoubles];

struct DeviceSetup {
  bool done = false;
  double* scratch = nullptr;   // device address of g_eigen_scratch on this device
  int grid = 0;                // co-resident blocks for k_jacobi
};
constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mutex;

// Once per device, with that device current: resolve the array's device
// address (the host-side symbol is only a stand-in) and size the cooperative
// grid.  The address belongs to the CUDA context current at that first call;
// a cudaDeviceReset of the device ends that context and leaves the cached
// address stale, so a process that resets a device must not call this entry
// point on it again.  A failed set-up caches nothing and the next call retries.
gbhf_status setup_device(int dev, DeviceSetup** out) {
  if (dev < 0 || dev >= kMaxDevices) return GBHF_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup& s = g_setup[dev];
  if (!s.done) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_eigen_scratch) != cudaSuccess || ptr == nullptr) return GBHF_ERR_CUDA;
    int nsm = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBHF_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gbhf::k_jacobi, 256, 0) != cudaSuccess)
      return GBHF_ERR_CUDA;
    // no resident block per SM: a cooperative launch could never start
    if (nsm < 1 || per_sm < 1) return GBHF_ERR_CUDA;
    s.scratch = static_cast<double*>(ptr);
    s.grid = nsm * (per_sm < 2 ? per_sm : 2);
    s.done = true;
  }
  *out = &s;
  return GBHF_OK;
}

}  // namespace

extern "C" gbhf_status gbhf_eigen_solve_noalloc(int n, const double* d_a, double* d_evals, double* d_evecs,
                                                void* stream) {
  if (n < 1 || n > kMaxN) return GBHF_ERR_BAD_INPUT;
  if (!d_a || !d_evals || !d_evecs) return GBHF_ERR_BAD_INPUT;
  // An error left pending by earlier runtime calls of this host thread (the
  // caller's own) is not this call's: clear it, so that the checks after the
  // launches below report only this call's failures.
  (void)cudaGetLastError();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBHF_ERR_NO_DEVICE;
  DeviceSetup* s = nullptr;
  gbhf_status st = setup_device(dev, &s);
  if (st != GBHF_OK) return st;
  cudaStream_t strm = static_cast<cudaStream_t>(stream);
  const int m = (n + (n & 1) < 2) ? 2 : n + (n & 1);   // even size, at most kMaxN
  double* base = s->scratch;
  unsigned* bar = reinterpret_cast<unsigned*>(base + kOffInts);   // [0] count, [1] generation
  int* status = reinterpret_cast<int*>(base + kOffInts + 1);
  int* sweeps = reinterpret_cast<int*>(base + kOffInts + 2);
  // the array keeps the previous call's contents: zero what must start at zero
  if (cudaMemsetAsync(base + kOffInts, 0, 3 * sizeof(double), strm) != cudaSuccess) return GBHF_ERR_CUDA;
  gbhf::k_jacobi_init<<<64, 256, 0, strm>>>(n, m, d_a, base + kOffA, base + kOffV);
  if (cudaGetLastError() != cudaSuccess) return GBHF_ERR_CUDA;
  gbhf::JacobiArgs a;
  a.n = n;
  a.m = m;
  a.A = base + kOffA;
  a.A2 = base + kOffA2;
  a.V = base + kOffV;
  a.rot = base + kOffRot;
  a.red = base + kOffRed;
  a.bar = bar;
  a.status = status;
  a.max_sweeps = 40;
  a.tol = 1e-14;
  a.sweeps_out = sweeps;
  const long work = (long)(m / 2) * (m / 2) + (long)n * (m / 2);
  int grid = (int)((work + 255) / 256);
  if (grid > s->grid) grid = s->grid;
  if (grid < 1) grid = 1;
  void* args[] = {&a};
  if (cudaLaunchCooperativeKernel((void*)gbhf::k_jacobi, dim3(grid), dim3(256), args, 0, strm) != cudaSuccess)
    return GBHF_ERR_CUDA;
  gbhf::k_sort_eig<<<1, 1024, 0, strm>>>(n, m, base + kOffA, base + kOffV, d_evals, d_evecs);
  if (cudaGetLastError() != cudaSuccess) return GBHF_ERR_CUDA;
  int hstatus = 0;
  if (cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, strm) != cudaSuccess)
    return GBHF_ERR_CUDA;
  if (cudaStreamSynchronize(strm) != cudaSuccess) return GBHF_ERR_CUDA;
  if (hstatus & GBHF_DEV_ERR_TIMEOUT) return GBHF_ERR_DEVICE_TIMEOUT;
  if (hstatus & GBHF_DEV_ERR_NOTCONV) return GBHF_ERR_NOT_CONVERGED;
  return GBHF_OK;
}
