// Allocation-free evaluation of the CCSD energy functional and residual norm.
//
// Some callers cannot call cudaMalloc at the point where they need the
// convergence test: a host framework that hands the GPU a fixed memory pool
// and forbids further allocation, or code running while a stream is being
// captured into a CUDA graph, where a cudaMalloc would break the capture.
// gbcc_energy_noalloc serves them: the caller passes every input and the
// output in its own device memory, and the per-pair partial sums live in a
// file-scope __device__ array instead of allocated scratch.
//
// The array holds one partial-sum record per virtual pair (a,b), so it bounds
// the problem size: v * v <= kMaxVirtualPairs (v <= 512), 8 MiB in total, reserved on
// every GPU that loads the library until the process exits.  All calls share
// it, and it keeps the last call's contents; every record a call reads is
// written earlier in the same call, so nothing needs clearing, but calls that
// overlap on the GPU (concurrent streams) race on it.  The first call on a
// device looks up the array's device address (cudaGetSymbolAddress), so make
// that first call before any stream capture begins.
#include <cmath>
#include <mutex>
#include <string>

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
  bool ready = false;
};
ScratchAddr g_addr[kMaxDevices];
std::mutex g_addr_mu;

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

// Device address of the scratch array on the current device (looked up once).
double* scratch_for_current_device(std::string& why) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    why = "no usable current CUDA device";
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_addr_mu);
  ScratchAddr& s = g_addr[dev];
  if (!s.ready) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_pair_partials);
    if (e != cudaSuccess || ptr == nullptr) {
      cudaGetLastError();
      why = std::string("cudaGetSymbolAddress of the energy scratch failed: ") + cudaGetErrorString(e);
      return nullptr;
    }
    s.partials = static_cast<double*>(ptr);
    s.ready = true;
  }
  return s.partials;
}

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
  std::string why;
  double* partials = scratch_for_current_device(why);
  if (!partials) {
    gbcc_set_thread_error("gbcc_energy_noalloc: " + why);
    return GBCC_ERR_CUDA;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
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
