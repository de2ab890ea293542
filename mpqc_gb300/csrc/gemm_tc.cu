// Split-BF16 tensor-core GEMM for sm_103a (tcgen05 + TMEM + TMA).
//
//   C[cm[m] + cn[n]] = beta * C + alpha * sum_{pairs (p,q)} sum_k A_p[m][k] B_q[n][k]
//
// A FP64 operand x is stored as BF16 slices x = x_0 + x_1 + x_2 (each slice the
// round-to-nearest BF16 of the remainder).  The product of two split operands
// is the sum of the slice products A_p B_q over the pairs with p + q below the
// slice count (the terms beneath the working precision are dropped, as in the
// error-free splitting of Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59,
// 95 (2012)).
//
// Accumulation.  The tensor core accumulates in FP32 and loses about one
// FP32 ulp of the running sum per MMA instruction, so a long K loop in one
// accumulator would lose accuracy in proportion to K.  Here every TMEM
// accumulation covers only a chunk of `chunk` k-blocks (4 * chunk MMAs).  The
// epilogue warps add each finished chunk to an FP32 register partial p and,
// every `fold` chunks, fold p into a float-float (hi + lo) accumulator kept in
// TMEM with Knuth's TwoSum; the error is that of one chunk plus `fold` FP32
// additions, independent of K.  TMEM holds two accumulators, so the MMAs of
// the next chunk run while the epilogue drains the previous one.
//
// With BN = 256 the two accumulators fill TMEM, so the chunks of a tile sum in
// FP32 registers only (error that of one chunk plus one FP32 addition per
// chunk); BN = 256 is about 1.5x faster, since an N = 128 MMA needs more shared-
// memory operand traffic per FLOP than the tensor core can be fed.
//
// Persistent kernel: one CTA per SM walks the 128 x BN output tiles
// (N-tile index fastest, so CTAs running together share the A panel in L2).
//   warp 0     : TMA producer (one thread), STAGES-deep smem ring
//   warp 1     : TMEM allocator + MMA issuer (one thread), kind::f16
//   warps 4..11: epilogue; warp w reads TMEM lanes 32*(w%4).. and the column
//                half (w-4)/4 of the tile (warps 2 and 3 only pad the
//                block to three warps per scheduler, which leaves 168
//                registers per thread for the float-float accumulators)
// Operand tiles are K-major with the 128-byte swizzle (TMA box 64 x rows).
// Every mbarrier wait is bounded: on timeout the kernel records kDevTimeout in
// *err, drains its own copies in flight, waits for its MMAs, frees its TMEM
// and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "fp_bits.cuh"
#include "kernels.h"

namespace gbcc {
namespace {

constexpr int BM = kTcBM;   // 128
constexpr int BK = kTcBK;   // 64 bf16 = 128 bytes = one swizzle row
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

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
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
// limit_ns, or early once any CTA has recorded an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const int* err,
                                          uint64_t limit_ns = kWaitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0) {
      if (globaltimer() - t0 > limit_ns) return false;
      if (*reinterpret_cast<const volatile int*>(err) != kDevOk) return false;
    }
  }
}

// Bounded wait that ignores the error word (teardown paths).
__device__ __forceinline__ void mbar_wait_teardown(uint64_t* bar, uint32_t parity) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(bar, parity) && globaltimer() - t0 < kWaitNs) {
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
// groups 1024 bytes apart (SBO), descriptor version 1, base offset 0 (tiles
// are 1024-byte aligned).
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
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}

__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// ---- CTA-pair (cta_group::2) helpers
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// shared::cluster address of the same shared variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t map_to_rank(const void* p, uint32_t rank) {
  uint32_t out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(smem_u32(p)), "r"(rank));
  return out;
}

__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc2(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc2(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// TMA load into this CTA's shared memory, completion counted on the mbarrier
// at cluster address `bar` (the pair leader's barrier).
__device__ __forceinline__ void tma_load_3d_pair(const CUtensorMap* map, uint32_t bar, void* dst, int c0, int c1,
                                                 int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void mma_bf16_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on the mbarrier at the same shared offset in every CTA of `mask`
// once the MMAs issued so far have completed.
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(mask)
      : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Knuth's TwoSum: hi + lo += x with the rounding error of hi + x kept in lo.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float v = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, v)), __fsub_rn(x, v));
  hi = s;
  lo = __fadd_rn(lo, e);
}

constexpr int kStgLd = 17;  // padded row of the per-warp output staging tile (8-byte words)

// SPS: slices per pipeline stage.  1: a stage holds one (A slice, B slice)
// pair of a k-block and feeds one pair of MMAs; 2: a stage holds both slices
// of A and of B of a k-block and feeds all three pair products (no tile is
// loaded twice; two slices only).
template <int BN, bool CTA2, int SPS = 1>
struct TcCfg {
  // a CTA pair splits B along N: each CTA stages BN/2 rows of it
  static constexpr int kBRows = CTA2 ? BN / 2 : BN;
  static constexpr uint32_t kABytes = BM * BK * 2;  // one slice tile
  static constexpr uint32_t kBBytes = kBRows * BK * 2;
  static constexpr uint32_t kAStage = SPS * kABytes;
  static constexpr uint32_t kBStage = SPS * kBBytes;
  static constexpr uint32_t kStageBytes = kAStage + kBStage;
  // warps 0 (TMA), 1 (MMA), 2-3 idle, 4-11 epilogue: three warps per
  // scheduler leave 168 registers a thread
  static constexpr int kEpiWarps = 8;
  static constexpr int kEpiWarp0 = 4;
  static constexpr int kThreads = 32 * (kEpiWarp0 + kEpiWarps);
  // staging tile per epilogue warp: (hi, lo) float pairs with the float-float
  // fold (BN <= 128), single floats at BN = 192 (room for a fifth stage, or two
  // stages of both slices), doubles at BN = 256.  The BN = 256 kernel spills
  // and keeps its spills in L1: enlarging its shared memory (a fourth stage)
  // measured 1.14 -> 0.88 PFLOP/s, so it keeps three stages.
  static constexpr uint32_t kStgElem = BN == 192 ? 4u : 8u;
  static constexpr uint32_t kStgBytes = kEpiWarps * 32 * kStgLd * kStgElem;
  // as many stages as fit in 227 KB next to the staging tile and barriers (one
  // pair per stage: 3 for BN = 256, 5 for 192 and 128, 7 for 64, 8 for 32; both
  // slices per stage: 2 for BN = 128 and 192)
  static constexpr int kStagesFit = static_cast<int>((232448u - 1024u - 256u - kStgBytes) / kStageBytes);
  static constexpr int kStages = kStagesFit > 8 ? 8 : kStagesFit;
  static_assert(kStages >= 2, "at least two pipeline stages");
  static_assert(SPS == 1 || !CTA2, "CTA pairs stage one slice pair");
  static constexpr uint32_t kSmem = 1024 + kStages * kStageBytes + kStgBytes + 256;
  // BN <= 128: two accumulators [0, 2 BN) + float-float words [2 BN, 4 BN);
  // BN = 256: the two accumulators fill TMEM and the chunks of a tile sum in
  // FP32 registers (no float-float fold)
  static constexpr bool kFold = BN <= 128;
  static_assert(BN % 32 == 0 && BN <= 256, "tile width");
  static constexpr uint32_t kTmemCols = BN >= 128 ? 512 : (BN >= 64 ? 256 : 128);
  static constexpr int kCols = BN / (kEpiWarps / 4);                // columns per epilogue thread
};

template <int BN, bool CTA2, int SPS>
__global__ void __launch_bounds__(TcCfg<BN, CTA2, SPS>::kThreads, 1)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const GemmTcArgs g) {
  using Cfg = TcCfg<BN, CTA2, SPS>;
  // CTA pair: rank 0 (leader) issues the MMAs for the 256-row tile; rank r
  // owns rows [128 r, 128 r + 128) of it and B rows [r BN/2, (r+1) BN/2)
  constexpr int BMP = CTA2 ? 2 * BM : BM;
  const uint32_t rank = CTA2 ? cluster_rank() : 0;
  const bool leader = rank == 0;
  const int unit = CTA2 ? static_cast<int>(blockIdx.x / 2) : static_cast<int>(blockIdx.x);
  const int nunits = CTA2 ? static_cast<int>(gridDim.x / 2) : static_cast<int>(gridDim.x);
  constexpr int S = Cfg::kStages;
  constexpr int COLS = Cfg::kCols;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + S * Cfg::kAStage;
  double* stg_all = reinterpret_cast<double*>(sB + S * Cfg::kBStage);
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + S * Cfg::kBStage + Cfg::kStgBytes);
  constexpr int kEpiWarps = Cfg::kEpiWarps;
  constexpr int kEpiWarp0 = Cfg::kEpiWarp0;
  uint64_t* empty = full + S;
  uint64_t* acc_full = empty + S;   // [2]
  uint64_t* acc_empty = acc_full + 2;  // [2]
  uint64_t* done = acc_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);

  const int warp = threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  const int ntn = static_cast<int>(g.Npad / BN);
  const int ntiles_mn = ntn * static_cast<int>(g.Mpad / BMP);
  const int ksplit = g.ksplit > 1 ? g.ksplit : 1;
  const int ntiles = ntiles_mn * ksplit;
  const int kblocks = static_cast<int>(g.Kpad / BK);
  const int kb_per_split = ksplit > 1 ? g.kb_per_split : kblocks;
  const int chunk = g.chunk > 0 ? g.chunk : 4;
  const int ntm = static_cast<int>(g.Mpad / BMP);
  const int group = g.group > 1 ? g.group : 1;
  // tile -> (K split, M block, N block); N fastest so CTAs running together
  // share the A panel in L2, or, with group > 1, bands of `group` M blocks
  // with N outer inside a band (fewer B columns live at once)
  auto decode = [&](int tile, int& m0, int& n0, int& kb0, int& n_iter, int& split) {
    split = tile / ntiles_mn;
    const int mn = tile - split * ntiles_mn;
    int mt, nt;
    if (group > 1) {
      const int band = mn / (group * ntn);
      const int rows = ntm - band * group < group ? ntm - band * group : group;
      const int idx = mn - band * group * ntn;
      mt = band * group + idx % rows;
      nt = idx / rows;
    } else {
      mt = mn / ntn;
      nt = mn - mt * ntn;
    }
    n0 = nt * BN;
    m0 = mt * BMP + static_cast<int>(rank) * BM;
    kb0 = split * kb_per_split;
    const int nkb = kblocks - kb0 < kb_per_split ? kblocks - kb0 : kb_per_split;
    n_iter = SPS == 1 ? nkb * g.npairs : nkb;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kEpiWarps * (CTA2 ? 2 : 1));
    }
    mbar_init(done, 1);
    fence_barrier_init();
  }
  if (warp == 1) {
    if constexpr (CTA2) tmem_alloc2(tmem_slot, Cfg::kTmemCols);
    else tmem_alloc(tmem_slot, Cfg::kTmemCols);
  }
  tc_fence_before();
  __syncthreads();
  if constexpr (CTA2) cluster_sync();  // both CTAs' barriers exist before any remote arrive
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // wait limit of the pipeline's barriers (a test hook may shorten it)
  const uint64_t wait_ns = g.wait_ns ? g.wait_ns : kWaitNs;

  if (warp == 0) {
    if (lane == 0) {
      prefetch_tmap(&tmA);
      prefetch_tmap(&tmB);
      // first panel row of the operands (a window of a larger panel); rows
      // past the panel's end load as zeros, rows past M or N are not stored
      const int a_row0 = static_cast<int>(g.a_row0), b_row0 = static_cast<int>(g.b_row0);
      uint32_t gi = 0;  // stage-use counter across tiles
      bool ok = true;
      // stage-ring position kept incrementally (no divisions in the loop)
      int s = 0;
      uint32_t ph = 0;
      const uint32_t full0 = CTA2 ? map_to_rank(&full[0], 0) : 0;
      for (int tile = unit; tile < ntiles && ok; tile += nunits) {
        int m0, n0, kb0, n_iter, split;
        decode(tile, m0, n0, kb0, n_iter, split);
        const int nb0 = n0 + static_cast<int>(rank) * Cfg::kBRows;
        int kb = kb0, pr = 0;
        for (int it = 0; it < n_iter; ++it, ++gi) {
          if (!mbar_wait(&empty[s], ph ^ 1, g.err, wait_ns)) {
            record_error(g.err, kDevTimeout);
            ok = false;
            break;
          }
          if constexpr (CTA2) {
            // the leader's full barrier counts the bytes of both CTAs
            const uint32_t bar = full0 + static_cast<uint32_t>(s) * 8u;
            if (leader) mbar_expect_tx(&full[s], 2 * Cfg::kStageBytes);
            tma_load_3d_pair(&tmA, bar, sA + s * Cfg::kAStage, 0, m0 + a_row0, g.pa[pr] * kblocks + kb);
            tma_load_3d_pair(&tmB, bar, sB + s * Cfg::kBStage, 0, nb0 + b_row0, g.pb[pr] * kblocks + kb);
          } else if constexpr (SPS == 1) {
            // test hook (gbcc_testing_gemm_timeout): leave one stage unloaded,
            // so that its consumer's bounded wait runs out
            if (g.skip_stage1 == 0 || static_cast<int64_t>(gi) + 1 != g.skip_stage1) {
              mbar_expect_tx(&full[s], Cfg::kStageBytes);
              tma_load_3d(&tmA, &full[s], sA + s * Cfg::kAStage, 0, m0 + a_row0, g.pa[pr] * kblocks + kb);
              tma_load_3d(&tmB, &full[s], sB + s * Cfg::kBStage, 0, nb0 + b_row0, g.pb[pr] * kblocks + kb);
            }
          } else {
            // every slice of A and B of this k-block
            mbar_expect_tx(&full[s], Cfg::kStageBytes);
#pragma unroll
            for (int j = 0; j < SPS; ++j) {
              tma_load_3d(&tmA, &full[s], sA + s * Cfg::kAStage + j * Cfg::kABytes, 0, m0 + a_row0,
                          j * kblocks + kb);
              tma_load_3d(&tmB, &full[s], sB + s * Cfg::kBStage + j * Cfg::kBBytes, 0, nb0 + b_row0,
                          j * kblocks + kb);
            }
          }
          if (SPS > 1 || ++pr == g.npairs) {
            pr = 0;
            ++kb;
          }
          if (++s == S) {
            s = 0;
            ph ^= 1;
          }
        }
      }
      // every copy issued here has landed before the CTA can exit: the
      // leader's full barriers count them; the partner sees them consumed
      const uint32_t first = gi > static_cast<uint32_t>(S) ? gi - S : 0;
      for (uint32_t u = first; u < gi; ++u) {
        if (leader) mbar_wait_teardown(&full[u % S], (u / S) & 1);
        else mbar_wait_teardown(&empty[u % S], (u / S) & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && leader) {
      constexpr uint32_t idesc = idesc_bf16(BMP, BN);
      uint32_t gi = 0;  // stage-use counter
      uint32_t c = 0;   // chunk counter
      bool ok = true;
      // shared-memory descriptors: built once, advanced by adding encoded
      // byte offsets (address >> 4) for the stage and the 16-element K step
      const uint64_t adesc0 = sdesc_sw128(smem_u32(sA));
      const uint64_t bdesc0 = sdesc_sw128(smem_u32(sB));
      int s = 0;
      uint32_t ph = 0;
      for (int tile = unit; tile < ntiles && ok; tile += nunits) {
        int m0, n0, kb0, n_iter, split;
        decode(tile, m0, n0, kb0, n_iter, split);
        int pos = 0;
        for (int it = 0; it < n_iter; ++it, ++gi) {
          const uint32_t b = c & 1;
          if (pos == 0 && !mbar_wait(&acc_empty[b], ((c >> 1) & 1) ^ 1, g.err, wait_ns)) {
            record_error(g.err, kDevTimeout);
            ok = false;
            break;
          }
          if (!mbar_wait(&full[s], ph, g.err, wait_ns)) {
            record_error(g.err, kDevTimeout);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + b * BN;
          if constexpr (SPS == 1) {
            const uint64_t ad = adesc0 + ((static_cast<uint64_t>(s) * Cfg::kAStage) >> 4);
            const uint64_t bd = bdesc0 + ((static_cast<uint64_t>(s) * Cfg::kBStage) >> 4);
#pragma unroll
            for (int k = 0; k < BK / 16; ++k) {
              const uint32_t acc = (pos > 0 || k > 0) ? 1u : 0u;
              if constexpr (CTA2) mma_bf16_pair(d, ad + 2 * k, bd + 2 * k, idesc, acc);
              else mma_bf16(d, ad + 2 * k, bd + 2 * k, idesc, acc);
            }
          } else {
            // all slice pairs of the k-block from the one stage
            for (int q = 0; q < g.npairs; ++q) {
              const uint64_t ad = adesc0 + ((static_cast<uint64_t>(s) * Cfg::kAStage +
                                             static_cast<uint64_t>(g.pa[q]) * Cfg::kABytes) >> 4);
              const uint64_t bd = bdesc0 + ((static_cast<uint64_t>(s) * Cfg::kBStage +
                                             static_cast<uint64_t>(g.pb[q]) * Cfg::kBBytes) >> 4);
#pragma unroll
              for (int k = 0; k < BK / 16; ++k) {
                const uint32_t acc = (pos > 0 || q > 0 || k > 0) ? 1u : 0u;
                mma_bf16(d, ad + 2 * k, bd + 2 * k, idesc, acc);
              }
            }
          }
          if constexpr (CTA2) mma_commit_pair(&empty[s], 0x3);
          else mma_commit(&empty[s]);
          if (++s == S) {
            s = 0;
            ph ^= 1;
          }
          if (++pos == chunk || it == n_iter - 1) {
            if constexpr (CTA2) mma_commit_pair(&acc_full[b], 0x3);
            else mma_commit(&acc_full[b]);
            ++c;
            pos = 0;
          }
        }
      }
      // TMEM is freed below only after every MMA issued here has completed
      if constexpr (CTA2) mma_commit_pair(done, 0x1);
      else mma_commit(done);
      mbar_wait_teardown(done, 0);
    }
  } else if (warp >= kEpiWarp0) {
    // epilogue warps
    const int q = warp & 3;
    const int h = (warp - kEpiWarp0) >> 2;
    const int row = q * 32 + lane;
    const int col0 = h * COLS;
    const uint32_t lane_addr = static_cast<uint32_t>(q * 32) << 16;
    // TMEM columns [2 BN, 3 BN): float-float high words, [3 BN, 4 BN): low words
    const uint32_t hi_base = tmem + lane_addr + 2 * BN + col0;
    const uint32_t lo_base = tmem + lane_addr + 3 * BN + col0;
    const int fold = g.fold > 0 ? g.fold : 16;
    uint32_t c = 0;
    bool ok = true;
    const uint32_t acc_empty_leader0 = CTA2 ? map_to_rank(&acc_empty[0], 0) : 0;
    const uint32_t acc_empty_leader1 = CTA2 ? map_to_rank(&acc_empty[1], 0) : 0;
    for (int tile = unit; tile < ntiles && ok; tile += nunits) {
      int m0i, n0i, kb0, n_iter, split;
      decode(tile, m0i, n0i, kb0, n_iter, split);
      const int64_t n0 = n0i, m0 = m0i;
      const int nchunks = (n_iter + chunk - 1) / chunk;
      // p: plain FP32 sum of the chunks since the last fold
      float p[COLS];
#pragma unroll
      for (int j = 0; j < COLS; ++j) p[j] = 0.f;
      bool first_fold = true;
      for (int cc = 0; cc < nchunks; ++cc, ++c) {
        const uint32_t b = c & 1;
        if (!mbar_wait(&acc_full[b], (c >> 1) & 1, g.err, wait_ns)) {
          record_error(g.err, kDevTimeout);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t base = tmem + lane_addr + b * BN + col0;
#pragma unroll
        for (int j0 = 0; j0 < COLS; j0 += 16) {
          uint32_t r[16];
          tmem_ld16(base + j0, r);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; ++j) p[j0 + j] = __fadd_rn(p[j0 + j], __uint_as_float(r[j]));
        }
        // the accumulator buffer is free again
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          if constexpr (CTA2) mbar_arrive_cluster(b ? acc_empty_leader1 : acc_empty_leader0);
          else mbar_arrive(&acc_empty[b]);
        }
        if (Cfg::kFold && ((cc + 1) % fold == 0 || cc == nchunks - 1)) {
          // fold p into the float-float (hi, lo) pair kept in TMEM
#pragma unroll
          for (int j0 = 0; j0 < COLS; j0 += 16) {
            uint32_t h[16], l[16];
            if (!first_fold) {
              tmem_ld16(hi_base + j0, h);
              tmem_ld16(lo_base + j0, l);
              tmem_ld_wait();
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              float hv = first_fold ? 0.f : __uint_as_float(h[j]);
              float lv = first_fold ? 0.f : __uint_as_float(l[j]);
              two_sum_acc(hv, lv, p[j0 + j]);
              h[j] = __float_as_uint(hv);
              l[j] = __float_as_uint(lv);
              p[j0 + j] = 0.f;
            }
            tmem_st16(hi_base + j0, h);
            tmem_st16(lo_base + j0, l);
          }
          tmem_st_wait();
          first_fold = false;
        }
      }
      if (!ok) break;
      if (*reinterpret_cast<const volatile int*>(g.err) != kDevOk) continue;
      if (ksplit == 1 && g.m_major) {
        // C contiguous in M: every lane owns one row, so the lanes of a warp
        // write 32 consecutive rows of one column
        const int64_t m = m0 + row;
#pragma unroll
        for (int j0 = 0; j0 < COLS; j0 += 16) {
          uint32_t h[16], l[16];
          if constexpr (Cfg::kFold) {
            tmem_ld16(hi_base + j0, h);
            tmem_ld16(lo_base + j0, l);
            tmem_ld_wait();
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              h[j] = __float_as_uint(p[j0 + j]);
              l[j] = 0u;
            }
          }
          if (m < g.M) {
            const int64_t om = g.cm[m];
            double cv[16];
            if (g.beta != 0.0) {
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const int64_t n = n0 + col0 + j0 + j;
                cv[j] = n < g.N ? g.C[om + g.cn[n]] : 0.0;
              }
            }
            if constexpr (Cfg::kFold) {
              // beta c + alpha (hi + lo): separate loops per beta, so no multiply by
              // beta is evaluated (as a select) where beta is 0 or 1
              if (g.beta == 0.0) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                  const int64_t n = n0 + col0 + j0 + j;
                  if (n < g.N)
                    g.C[om + g.cn[n]] = g.alpha * (f2d_exact(__uint_as_float(h[j])) + f2d_exact(__uint_as_float(l[j])));
                }
              } else if (g.beta == 1.0) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                  const int64_t n = n0 + col0 + j0 + j;
                  if (n < g.N)
                    g.C[om + g.cn[n]] = fma(g.alpha, f2d_exact(__uint_as_float(h[j])),
                                            fma(g.alpha, f2d_exact(__uint_as_float(l[j])), cv[j]));
                }
              } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                  const int64_t n = n0 + col0 + j0 + j;
                  if (n < g.N)
                    g.C[om + g.cn[n]] = fma(g.alpha, f2d_exact(__uint_as_float(h[j])),
                                            fma(g.alpha, f2d_exact(__uint_as_float(l[j])), g.beta * cv[j]));
                }
              }
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const int64_t n = n0 + col0 + j0 + j;
                if (n < g.N) {
                  const double val = g.alpha * (static_cast<double>(__uint_as_float(h[j])) +
                                                static_cast<double>(__uint_as_float(l[j])));
                  g.C[om + g.cn[n]] = (g.beta == 0.0) ? val : fma(g.beta, cv[j], val);
                }
              }
            }
          }
        }
        continue;
      }
      // stage 32 rows x 16 columns through shared memory, then write with the
      // lanes along N (coalesced when C is contiguous in N)
      uint8_t* stg_w = reinterpret_cast<uint8_t*>(stg_all) + (warp - kEpiWarp0) * 32 * kStgLd * Cfg::kStgElem;
      double* stg = reinterpret_cast<double*>(stg_w);  // float-float variants: read as float2
      float* stgf = reinterpret_cast<float*>(stg_w);   // FP32 variants
      const int cj = lane & 15;
#pragma unroll
      for (int j0 = 0; j0 < COLS; j0 += 16) {
        uint32_t h[16], l[16];
        if constexpr (Cfg::kFold) {
          tmem_ld16(hi_base + j0, h);
          tmem_ld16(lo_base + j0, l);
          tmem_ld_wait();
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            h[j] = __float_as_uint(p[j0 + j]);
            l[j] = 0u;
          }
        }
        if constexpr (Cfg::kFold) {
          // (hi, lo) pairs, converted to FP64 at the store
          float2* stg2 = reinterpret_cast<float2*>(stg);
#pragma unroll
          for (int j = 0; j < 16; ++j)
            stg2[lane * kStgLd + j] = make_float2(__uint_as_float(h[j]), __uint_as_float(l[j]));
        } else if constexpr (Cfg::kStgElem == 4) {
#pragma unroll
          for (int j = 0; j < 16; ++j) stgf[lane * kStgLd + j] = __uint_as_float(h[j]);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j)
            stg[lane * kStgLd + j] =
                static_cast<double>(__uint_as_float(h[j])) + static_cast<double>(__uint_as_float(l[j]));
        }
        __syncwarp();
        const int64_t n = n0 + col0 + j0 + cj;
        if (ksplit > 1) {
          // K-split partial tile: plain stores, reduced by splitk_reduce
          double* P = g.partial + static_cast<int64_t>(split) * g.Mpad * g.Npad + n;
#pragma unroll
          for (int rr = lane >> 4; rr < 32; rr += 2) {
            const int64_t m = m0 + q * 32 + rr;
            if constexpr (Cfg::kFold) {
              const float2 hl = reinterpret_cast<const float2*>(stg)[rr * kStgLd + cj];
              P[m * g.Npad] = f2d_exact(hl.x) + f2d_exact(hl.y);
            } else if constexpr (Cfg::kStgElem == 4) {
              P[m * g.Npad] = static_cast<double>(stgf[rr * kStgLd + cj]);
            } else {
              P[m * g.Npad] = stg[rr * kStgLd + cj];
            }
          }
        } else if (cj < COLS && n < g.N) {
          const int64_t on = g.cn[n];
          // 16 rows per lane: issue every read of C before the stores
          double cv[16];
          int64_t off[16];
#pragma unroll
          for (int r = 0; r < 16; ++r) {
            const int64_t m = m0 + q * 32 + (lane >> 4) + 2 * r;
            off[r] = m < g.M ? g.cm[m] + on : -1;
          }
          if (g.beta != 0.0) {
#pragma unroll
            for (int r = 0; r < 16; ++r) cv[r] = off[r] >= 0 ? g.C[off[r]] : 0.0;
          }
          if constexpr (Cfg::kFold) {
            const float2* stg2 = reinterpret_cast<const float2*>(stg);
            if (g.beta == 0.0) {
#pragma unroll
              for (int r = 0; r < 16; ++r) {
                if (off[r] < 0) continue;
                const float2 hl = stg2[((lane >> 4) + 2 * r) * kStgLd + cj];
                g.C[off[r]] = g.alpha * (f2d_exact(hl.x) + f2d_exact(hl.y));
              }
            } else if (g.beta == 1.0) {
#pragma unroll
              for (int r = 0; r < 16; ++r) {
                if (off[r] < 0) continue;
                const float2 hl = stg2[((lane >> 4) + 2 * r) * kStgLd + cj];
                g.C[off[r]] = fma(g.alpha, f2d_exact(hl.x), fma(g.alpha, f2d_exact(hl.y), cv[r]));
              }
            } else {
#pragma unroll
              for (int r = 0; r < 16; ++r) {
                if (off[r] < 0) continue;
                const float2 hl = stg2[((lane >> 4) + 2 * r) * kStgLd + cj];
                g.C[off[r]] = fma(g.alpha, f2d_exact(hl.x), fma(g.alpha, f2d_exact(hl.y), g.beta * cv[r]));
              }
            }
          } else {
#pragma unroll
            for (int r = 0; r < 16; ++r) {
              if (off[r] < 0) continue;
              double sv;
              if constexpr (Cfg::kStgElem == 4) sv = static_cast<double>(stgf[((lane >> 4) + 2 * r) * kStgLd + cj]);
              else sv = stg[((lane >> 4) + 2 * r) * kStgLd + cj];
              const double val = g.alpha * sv;
              g.C[off[r]] = (g.beta == 0.0) ? val : fma(g.beta, cv[r], val);
            }
          }
        }
        __syncwarp();
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if constexpr (CTA2) {
    __syncwarp();
    cluster_sync();  // no remote arrive or MMA into this CTA is pending
  }
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    if constexpr (CTA2) tmem_dealloc2(tmem, Cfg::kTmemCols);
    else tmem_dealloc(tmem, Cfg::kTmemCols);
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

// Operand panels are k-block major per slice, [Kpad/64][rows][64] BF16, so a
// box of 64 K elements x box_rows rows is one contiguous run; the slice
// stride is (Kpad/64) times the k-block stride, so (k-block, slice) fold into
// the third coordinate: slice * (Kpad/64) + k-block.
bool make_map(CUtensorMap* map, const void* base, int64_t slices, int64_t rows, int64_t kpad,
              int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {static_cast<cuuint64_t>(BK), static_cast<cuuint64_t>(rows),
                        static_cast<cuuint64_t>(slices * (kpad / BK))};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(BK * 2), static_cast<cuuint64_t>(rows * BK * 2)};
  cuuint32_t box[3] = {static_cast<cuuint32_t>(BK), static_cast<cuuint32_t>(box_rows), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}


template <int BN, bool CTA2, int SPS = 1>
bool launch_bn(const GemmTcArgs& g, cudaStream_t st) {
  using Cfg = TcCfg<BN, CTA2, SPS>;
  CUtensorMap ma, mb;
  if (!make_map(&ma, g.A, g.a_slices, g.a_rows ? g.a_rows : g.Mpad, g.Kpad, BM)) return false;
  if (!make_map(&mb, g.B, g.b_slices, g.b_rows ? g.b_rows : g.Npad, g.Kpad, Cfg::kBRows)) return false;
  // once per instantiation; the initialisation of a function-local static is
  // thread-safe, so concurrent solves (gbcc_solve_batch) may reach it together
  static const bool attr_set = cudaFuncSetAttribute(gemm_tc_kernel<BN, CTA2, SPS>,
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    Cfg::kSmem) == cudaSuccess;
  if (!attr_set) return false;
  const int64_t units = (g.Npad / BN) * (g.Mpad / (CTA2 ? 2 * BM : BM)) * (g.ksplit > 1 ? g.ksplit : 1);
  if (!CTA2) {
    const int grid = static_cast<int>(units < num_sms() ? units : num_sms());
    gemm_tc_kernel<BN, false, SPS><<<grid, Cfg::kThreads, Cfg::kSmem, st>>>(ma, mb, g);
    return true;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(Cfg::kThreads);
  cfg.dynamicSmemBytes = Cfg::kSmem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  static const int max_pairs = [&cfg] {
    cfg.gridDim = dim3(2 * (num_sms() / 2));
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, gemm_tc_kernel<BN, true, 1>, &cfg) != cudaSuccess || n < 1) {
      cudaGetLastError();
      n = num_sms() / 2;
    }
    return n;
  }();
  const int64_t pairs = units < max_pairs ? units : max_pairs;
  cfg.gridDim = dim3(static_cast<unsigned>(2 * pairs));
  return cudaLaunchKernelEx(&cfg, gemm_tc_kernel<BN, true, 1>, ma, mb, g) == cudaSuccess;
}

}  // namespace

int gemm_tc_pick_bn(int64_t N, bool allow256) {
  if (N <= 32) return 32;
  if (N <= 64) return 64;
  if (allow256 && N >= 256) {
    // 256- or 192-wide tiles, whichever pads N less (e.g. 528 = 3 x 176 -> 576 vs 768)
    const int64_t p256 = (N + 255) / 256 * 256, p192 = (N + 191) / 192 * 192;
    return p192 < p256 ? 192 : 256;
  }
  return 128;
}

int gemm_tc_bn_candidates(int64_t N, bool allow256, int* out) {
  int n = 0;
  const int first = gemm_tc_pick_bn(N, allow256);
  out[n++] = first;
  auto add = [&](int bn) {
    for (int i = 0; i < n; ++i)
      if (out[i] == bn) return;
    out[n++] = bn;
  };
  if (N > 32) add(N <= 64 ? 32 : 64);
  if (N > 64) add(128);
  if (allow256 && N >= 256) {
    add(192);
    add(256);
  }
  return n;
}

bool launch_gemm_tc(const GemmTcArgs& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return true;
  if (g.Mpad % BM || g.Kpad % BK || g.Kpad < BK || g.Npad % g.bn || g.npairs < 1 ||
      g.npairs > kMaxPairs)
    return false;
  if (g.Mpad > (1LL << 31) - 1 || g.Npad > (1LL << 31) - 1 || g.Kpad > (1LL << 31) - 1) return false;
  if ((g.a_rows && g.a_rows < g.Mpad) || (g.b_rows && g.b_rows < g.Npad)) return false;
  if (g.a_row0 < 0 || g.b_row0 < 0 || g.a_row0 + g.Mpad > (1LL << 31) - 1 || g.b_row0 + g.Npad > (1LL << 31) - 1)
    return false;
  if ((g.Npad / g.bn) * (g.Mpad / BM) * (g.ksplit > 1 ? g.ksplit : 1) > (1LL << 31) - 1) return false;
  if (g.ksplit > 1 && (!g.partial || g.kb_per_split < 1 ||
                       static_cast<int64_t>(g.ksplit - 1) * g.kb_per_split >= g.Kpad / BK))
    return false;
  if (g.cta2) {
    if (g.Mpad % (2 * BM)) return false;
    switch (g.bn) {
      case 64: return launch_bn<64, true>(g, st);
      case 128: return launch_bn<128, true>(g, st);
      default: return false;
    }
  }
  if (g.sps == 2) {
    // both slices per stage: two slices, every pair (p, q) with p, q < 2
    if (g.a_slices != 2 || g.b_slices != 2) return false;
    for (int q = 0; q < g.npairs; ++q)
      if (g.pa[q] > 1 || g.pb[q] > 1) return false;
    // one TMEM accumulation spans the same number of MMAs as with one pair
    // per stage: chunk counts stages
    GemmTcArgs h = g;
    h.chunk = std::max(1, (g.chunk > 0 ? g.chunk : 4) / g.npairs);
    switch (g.bn) {
      case 64: return launch_bn<64, false, 2>(h, st);
      case 128: return launch_bn<128, false, 2>(h, st);
      case 192: return launch_bn<192, false, 2>(h, st);
      default: return false;
    }
  }
  switch (g.bn) {
    case 32: return launch_bn<32, false>(g, st);
    case 64: return launch_bn<64, false>(g, st);
    case 128: return launch_bn<128, false>(g, st);
    case 192: return launch_bn<192, false>(g, st);
    case 256: return launch_bn<256, false>(g, st);
    default: return false;
  }
}

}  // namespace gbcc
