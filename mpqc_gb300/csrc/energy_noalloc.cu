// Allocation-free evaluation of the CCSD energy functional and residual norm.
//
// Some callers cannot call cudaMalloc at the point where they need the
// convergence test.  A host framework may hand the GPU one fixed memory pool
// at start-up and forbid any later allocation (MPQC-style drivers that size
// the device pool to the integrals they keep resident), and cudaMalloc may
// synchronise the whole device, which a caller overlapping the test with work
// on other streams cannot afford.  gbcc_energy_noalloc serves them: the caller
// passes every input and the output in its own device memory, and the
// per-pair partial sums live in a file-scope __device__ array instead of
// allocated scratch.
//
// The array holds one partial-sum record per virtual pair (a,b), so it bounds
// the problem size: v * v <= kMaxVirtualPairs (v <= 512), 8 MiB in total, reserved on
// every GPU that loads the library until the process exits.  All calls share
// it, and it keeps the last call's contents; every record a call reads is
// written earlier in the same call, so nothing needs clearing, but calls that
// overlap on the GPU (concurrent streams) race on it.  The first call on a
// device (in each CUDA context of that device, e.g. again after a
// cudaDeviceReset) looks up the array's device address with
// cudaGetSymbolAddress, with the stream's device current; make that first call
// before any stream capture begins.
#include <cmath>
#include <mutex>
#include <string>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "../../include/gbcc.h"
#include "engine.h"

namespace gbcc {
namespace {

constexpr int64_t kMaxVirtualPairs = 512 * 512;  // v <= 512
constexpr int kNoAllocThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_pair_partials[kMaxVirtualPairs * 4];

struct ScratchAddr {
  double* partials = nullptr;
  CUcontext ctx = nullptr;  // context the address belongs to
};
ScratchAddr g_addr[kMaxDevices];
std::mutex g_addr_mu;

// cuCtxGetCurrent through the runtime's driver entry point (no libcuda link)
PFN_cuCtxGetCurrent_v4000 ctx_get_current_fn() {
  static PFN_cuCtxGetCurrent_v4000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
  }();
  return fn;
}

__device__ __forceinline__ double block_sum_na(double v, double* sh) {
  const int tid = threadIdx.x;
  sh[tid] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] += sh[tid + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Block p sums the (a,b) = p slice of the doubles terms and a strided share
// of the singles terms:
//   [0] sum r1^2  [1] sum r2^2  [2] sum (f_ai + r1) t1
//   [3] sum (g_abij + r2)(2 tau(a,b,i,j) - tau(b,a,i,j))
__global__ void __launch_bounds__(kNoAllocThreads)
    pair_partials_kernel(int64_t o, int64_t v, const double* __restrict__ f_ai,
                         const double* __restrict__ g_abij, const double* __restrict__ t1,
                         const double* __restrict__ tau, const double* __restrict__ r1,
                         const double* __restrict__ r2, double* __restrict__ partials) {
  __shared__ double sh[kNoAllocThreads];
  const int64_t p = blockIdx.x;
  const int64_t o2 = o * o;
  const int64_t a = p / v, b = p % v;
  const double* r2p = r2 + p * o2;
  const double* gp = g_abij + p * o2;
  const double* tp = tau + p * o2;
  const double* tq = tau + (b * v + a) * o2;
  double s_r1 = 0.0, s_r2 = 0.0, s_e1 = 0.0, s_e2 = 0.0;
  for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
    const double r = r2p[ij];
    s_r2 = fma(r, r, s_r2);
    s_e2 = fma(gp[ij] + r, 2.0 * tp[ij] - tq[ij], s_e2);
  }
  const int64_t n1 = v * o;
  for (int64_t e = p * blockDim.x + threadIdx.x; e < n1; e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double r = r1[e];
    s_r1 = fma(r, r, s_r1);
    s_e1 = fma(f_ai[e] + r, t1[e], s_e1);
  }
  s_r1 = block_sum_na(s_r1, sh);
  s_r2 = block_sum_na(s_r2, sh);
  s_e1 = block_sum_na(s_e1, sh);
  s_e2 = block_sum_na(s_e2, sh);
  if (threadIdx.x == 0) {
    partials[p * 4 + 0] = s_r1;
    partials[p * 4 + 1] = s_r2;
    partials[p * 4 + 2] = s_e1;
    partials[p * 4 + 3] = s_e2;
  }
}

// One block: fixed-order sum of the npairs records, then
// out[0] = E = 2 s_e1 + s_e2, out[1] = sqrt(s_r1 + s_r2) / (n1 + n2).
__global__ void __launch_bounds__(kNoAllocThreads)
    pair_reduce_kernel(int64_t npairs, double denom, const double* __restrict__ partials, double* out) {
  __shared__ double sh[kNoAllocThreads];
  double s[4];
  for (int q = 0; q < 4; ++q) {
    double acc = 0.0;
    for (int64_t p = threadIdx.x; p < npairs; p += blockDim.x) acc += partials[p * 4 + q];
    s[q] = block_sum_na(acc, sh);
  }
  if (threadIdx.x == 0) {
    out[0] = 2.0 * s[2] + s[3];
    out[1] = sqrt(s[0] + s[1]) / denom;
  }
}

// Device address of the scratch array on device `dev`, which the caller has
// made current.  Looked up once per device and context: a new primary
// context (after cudaDeviceReset) reloads the module, so the address is
// looked up again when the current context is not the one it came from.
double* scratch_for_device(int dev, std::string& why) {
  if (dev < 0 || dev >= kMaxDevices) {
    why = "device ordinal out of range";
    return nullptr;
  }
  CUcontext ctx = nullptr;
  if (auto fn = ctx_get_current_fn()) {
    if (fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  }
  std::lock_guard<std::mutex> lock(g_addr_mu);
  ScratchAddr& s = g_addr[dev];
  if (!s.partials || ctx == nullptr || s.ctx != ctx) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_pair_partials);
    if (e != cudaSuccess || ptr == nullptr) {
      cudaGetLastError();
      why = std::string("cudaGetSymbolAddress of the energy scratch failed: ") + cudaGetErrorString(e);
      return nullptr;
    }
    s.partials = static_cast<double*>(ptr);
    s.ctx = ctx;
  }
  return s.partials;
}

// Device memory of device `dev` (or managed memory): anything else, such as a
// host pointer, would reach the kernels as a bad address.
bool device_pointer_on(const void* p, int dev) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

// Makes `dev` current for its lifetime and restores the caller's device.
struct DeviceScope {
  int prev = -1;
  bool ok = false;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    ok = cudaSetDevice(dev) == cudaSuccess;
    if (!ok) cudaGetLastError();
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace
}  // namespace gbcc

void gbcc_set_thread_error(const std::string& msg);  // api.cpp

extern "C" gbcc_status gbcc_energy_noalloc(int64_t o, int64_t v, const double* f_ai, const double* g_abij,
                                           const double* t1_ai, const double* tau_abij, const double* r1_ai,
                                           const double* r2_abij, double* out, void* stream) {
  using namespace gbcc;
  if (o < 1 || v < 1) {
    gbcc_set_thread_error("gbcc_energy_noalloc: o and v must be >= 1");
    return GBCC_ERR_INVALID_ARG;
  }
  if (v > 512 || v * v > kMaxVirtualPairs) {
    gbcc_set_thread_error("gbcc_energy_noalloc: v = " + std::to_string(v) +
                          " exceeds the allocation-free limit v <= 512 (use gbcc_energy)");
    return GBCC_ERR_INVALID_ARG;
  }
  if (!f_ai || !g_abij || !t1_ai || !tau_abij || !r1_ai || !r2_abij || !out) {
    gbcc_set_thread_error("gbcc_energy_noalloc: NULL argument");
    return GBCC_ERR_INVALID_ARG;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = -1;
  if (cudaStreamGetDevice(st, &dev) != cudaSuccess || dev < 0) {
    cudaGetLastError();
    gbcc_set_thread_error("gbcc_energy_noalloc: cannot determine the stream's device");
    return GBCC_ERR_INVALID_ARG;
  }
  const void* ptrs[] = {f_ai, g_abij, t1_ai, tau_abij, r1_ai, r2_abij, out};
  const char* names[] = {"f_ai", "g_abij", "t1", "tau", "r1", "r2", "out"};
  for (int k = 0; k < 7; ++k)
    if (!device_pointer_on(ptrs[k], dev)) {
      gbcc_set_thread_error(std::string("gbcc_energy_noalloc: ") + names[k] +
                            " is not device memory of the stream's device " + std::to_string(dev));
      return GBCC_ERR_INVALID_ARG;
    }
  DeviceScope scope(dev);
  if (!scope.ok) {
    gbcc_set_thread_error("gbcc_energy_noalloc: cannot make the stream's device current");
    return GBCC_ERR_CUDA;
  }
  std::string why;
  double* partials = scratch_for_device(dev, why);
  if (!partials) {
    gbcc_set_thread_error("gbcc_energy_noalloc: " + why);
    return GBCC_ERR_CUDA;
  }
  const int64_t npairs = v * v;
  pair_partials_kernel<<<static_cast<unsigned>(npairs), kNoAllocThreads, 0, st>>>(
      o, v, f_ai, g_abij, t1_ai, tau_abij, r1_ai, r2_abij, partials);
  pair_reduce_kernel<<<1, kNoAllocThreads, 0, st>>>(npairs, static_cast<double>(v * o + npairs * o * o),
                                                    partials, out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    gbcc_set_thread_error(std::string("gbcc_energy_noalloc: launch failed: ") + cudaGetErrorString(e));
    return GBCC_ERR_CUDA;
  }
  return GBCC_OK;
}
