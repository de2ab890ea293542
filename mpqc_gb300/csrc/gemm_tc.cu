// Split-BF16 tensor-core GEMM for sm_103a (tcgen05 + TMEM + TMA).
//
//   C[cm[m] + cn[n]] = beta * C + alpha * sum_{pairs (p,q)} sum_k A_p[m][k] B_q[n][k]
//
// A FP64 operand x is stored as BF16 slices x = x_0 + x_1 + x_2 (each slice the
// round-to-nearest BF16 of the remainder).  The product of two split operands
// is the sum of the slice products A_p B_q over the chosen pairs (p + q below
// the slice count drops the terms beneath the working precision, as in the
// Ozaki splitting of Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59 (2012)).
// All slice products accumulate into one FP32 TMEM accumulator; the epilogue
// converts to FP64 and scatters through the output offset tables.
//
// Pipeline (one 128 x BN output tile per CTA, 6 warps):
//   warp 0     : TMA producer (one thread) -> STAGES-deep smem ring
//   warp 1     : TMEM allocator + MMA issuer (one thread), tcgen05.mma kind::f16
//   warps 2..5 : epilogue, tcgen05.ld 32x32b (warp w reads TMEM lanes 32*(w%4)...)
// Operand tiles are K-major with the 128-byte swizzle (TMA box 64 x rows).
// Every mbarrier wait is bounded: on timeout the kernel records kDevTimeout in
// *err, drains its own copies in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels.h"

namespace gbcc {
namespace {

constexpr int BM = kTcBM;   // 128
constexpr int BK = kTcBK;   // 64 bf16 = 128 bytes = one swizzle row
constexpr int kThreadsTc = 192;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of `parity` to complete.  Gives up (false) after
// kWaitNs, or early once another CTA has recorded an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0) {
      if (globaltimer() - t0 > kWaitNs) return false;
      if (*reinterpret_cast<const volatile int*>(err) != kDevOk) return false;
    }
  }
}

__device__ __forceinline__ void record_error(int* err, int code) { atomicCAS(err, kDevOk, code); }

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_3d(const CUtensorMap* map, uint64_t* bar, void* dst, int c0,
                                            int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// Shared-memory matrix descriptor: K-major tile, 128-byte swizzle, 8-row
// groups 1024 bytes apart (SBO), version 1, base offset 0 (tiles are
// 1024-byte aligned).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(16u >> 4) << 16;    // leading byte offset (unused for SW128 K-major)
  d |= static_cast<uint64_t>(1024u >> 4) << 32;  // stride byte offset
  d |= static_cast<uint64_t>(1) << 46;           // descriptor version
  d |= static_cast<uint64_t>(2) << 61;           // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int BN>
struct TcCfg {
  static constexpr int kStages = (BN >= 256) ? 4 : (BN >= 128 ? 6 : 8);
  static constexpr uint32_t kABytes = BM * BK * 2;
  static constexpr uint32_t kBBytes = BN * BK * 2;
  static constexpr uint32_t kStageBytes = kABytes + kBBytes;
  static constexpr uint32_t kSmem = 1024 + kStages * kStageBytes + 256;
  static constexpr uint32_t kTmemCols = BN < 32 ? 32 : BN;
};

template <int BN>
__global__ void __launch_bounds__(kThreadsTc, 1)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const GemmTcArgs g) {
  using Cfg = TcCfg<BN>;
  constexpr int S = Cfg::kStages;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + S * Cfg::kABytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + S * Cfg::kBBytes);
  uint64_t* empty = full + S;
  uint64_t* accb = empty + S;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accb + 1);

  const int warp = threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  const int64_t n0 = static_cast<int64_t>(blockIdx.x) * BN;
  const int64_t m0 = static_cast<int64_t>(blockIdx.y) * BM;
  const int kblocks = static_cast<int>(g.Kpad / BK);
  const int n_iter = kblocks * g.npairs;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accb, 1);
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, Cfg::kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      prefetch_tmap(&tmA);
      prefetch_tmap(&tmB);
      int issued = 0;
      for (int it = 0; it < n_iter; ++it) {
        const int s = it % S;
        const uint32_t ph = (it / S) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1, g.err)) {
          record_error(g.err, kDevTimeout);
          break;
        }
        const int kb = it / g.npairs;
        const int pr = it % g.npairs;
        mbar_expect_tx(&full[s], Cfg::kStageBytes);
        tma_load_3d(&tmA, &full[s], sA + s * Cfg::kABytes, kb * BK, static_cast<int>(m0), g.pa[pr]);
        tma_load_3d(&tmB, &full[s], sB + s * Cfg::kBBytes, kb * BK, static_cast<int>(n0), g.pb[pr]);
        ++issued;
      }
      // drain: every copy this thread issued has landed before the CTA exits
      const int first = issued > S ? issued - S : 0;
      for (int it = first; it < issued; ++it) {
        if (!mbar_wait(&full[it % S], (it / S) & 1, g.err)) {
          // last resort: bounded again, ignoring the error early-exit
          const uint64_t t0 = globaltimer();
          while (!mbar_try_wait(&full[it % S], (it / S) & 1) && globaltimer() - t0 < kWaitNs) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(BM, BN);
      bool ok = true;
      for (int it = 0; it < n_iter; ++it) {
        const int s = it % S;
        const uint32_t ph = (it / S) & 1;
        if (!mbar_wait(&full[s], ph, g.err)) {
          record_error(g.err, kDevTimeout);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(sA + s * Cfg::kABytes);
        const uint32_t b0 = smem_u32(sB + s * Cfg::kBBytes);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          mma_bf16(tmem, sdesc_sw128(a0 + k * 32), sdesc_sw128(b0 + k * 32), idesc,
                   (it > 0 || k > 0) ? 1u : 0u);
        }
        mma_commit(&empty[s]);
      }
      (void)ok;
      mma_commit(accb);  // tracks completion of every MMA issued above
      // TMEM is freed below only after every issued MMA has completed
      const uint64_t t0 = globaltimer();
      while (!mbar_try_wait(accb, 0) && globaltimer() - t0 < kWaitNs) {
      }
    }
  } else {
    // epilogue warps 2..5
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const int64_t m = m0 + row;
    const bool ready = mbar_wait(accb, 0, g.err);
    tc_fence_after();
    const bool write = ready && (*reinterpret_cast<const volatile int*>(g.err) == kDevOk);
    if (!ready) record_error(g.err, kDevTimeout);
    if (ready) {
      const int64_t om = (m < g.M) ? g.cm[m] : 0;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(c0), r);
        if (write && m < g.M) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int64_t n = n0 + c0 + j;
            if (n < g.N) {
              double* p = g.C + om + g.cn[n];
              const double val = g.alpha * static_cast<double>(__uint_as_float(r[j]));
              *p = (g.beta == 0.0) ? val : fma(g.beta, *p, val);
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, Cfg::kTmemCols);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool make_map(CUtensorMap* map, const void* base, int64_t slices, int64_t rows, int64_t kpad,
              int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {static_cast<cuuint64_t>(kpad), static_cast<cuuint64_t>(rows),
                        static_cast<cuuint64_t>(slices)};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(kpad * 2), static_cast<cuuint64_t>(rows * kpad * 2)};
  cuuint32_t box[3] = {static_cast<cuuint32_t>(BK), static_cast<cuuint32_t>(box_rows), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int BN>
bool launch_bn(const GemmTcArgs& g, cudaStream_t st) {
  using Cfg = TcCfg<BN>;
  CUtensorMap ma, mb;
  if (!make_map(&ma, g.A, g.a_slices, g.Mpad, g.Kpad, BM)) return false;
  if (!make_map(&mb, g.B, g.b_slices, g.Npad, g.Kpad, BN)) return false;
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(gemm_tc_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             Cfg::kSmem) != cudaSuccess)
      return false;
    attr_set = true;
  }
  dim3 grid(static_cast<unsigned>(g.Npad / BN), static_cast<unsigned>(g.Mpad / BM));
  gemm_tc_kernel<BN><<<grid, kThreadsTc, Cfg::kSmem, st>>>(ma, mb, g);
  return true;
}

}  // namespace

int gemm_tc_pick_bn(int64_t N) {
  if (N <= 32) return 32;
  if (N <= 64) return 64;
  if (N <= 128) return 128;
  return 256;
}

bool launch_gemm_tc(const GemmTcArgs& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return true;
  if (g.Mpad % BM || g.Kpad % BK || g.Npad % g.bn || g.npairs < 1 || g.npairs > kMaxPairs) return false;
  if (g.Mpad > (1LL << 31) - 1 || g.Npad > (1LL << 31) - 1 || g.Kpad > (1LL << 31) - 1) return false;
  if (g.Mpad / BM > 65535) return false;
  switch (g.bn) {
    case 32: return launch_bn<32>(g, st);
    case 64: return launch_bn<64>(g, st);
    case 128: return launch_bn<128>(g, st);
    case 256: return launch_bn<256>(g, st);
    default: return false;
  }
}

}  // namespace gbcc
