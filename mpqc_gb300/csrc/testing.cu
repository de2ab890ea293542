// Test hooks (include/gbcc_testing.h): single-kernel GEMM runs and an FP64
// throughput probe.  Not used by the solver itself.
#include <cstdio>
#include <vector>

#include "../../include/gbcc.h"
#include "../../include/gbcc_testing.h"
#include "engine.h"
#include "kernels.h"

namespace {

int64_t rup(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

__global__ void fp64_fma_probe(double* out, int iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double m = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) out[0] = s;  // keeps the loop alive
}

// FP64 tensor-core (DMMA) throughput: each warp issues
// mma.sync.aligned.m8n8k4.row.col.f64 (512 FLOP) on register operands, four
// independent accumulators deep.
__global__ void fp64_dmma_probe(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-9, b = 0.999999;
  double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(c[2 * j]), "+d"(c[2 * j + 1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
  for (int j = 0; j < 8; ++j) s += c[j];
  if (s == 12345.678) out[0] = s;  // keeps the loop alive
}

}  // namespace

extern "C" int gbcc_testing_gemm(int64_t M, int64_t N, int64_t K, const double* A, const double* B,
                                 double* Cout, int slices, int repeat, float* ms) {
  return gbcc_testing_gemm_ex(M, N, K, A, B, Cout, slices, 1, 0, 0, 0, 0, repeat, ms);
}

extern "C" int gbcc_testing_gemm_ex(int64_t M, int64_t N, int64_t K, const double* A, const double* B,
                                    double* Cout, int slices, int ksplit, int bn_req, int cta2, int chunk,
                                    int fold, int repeat, float* ms) {
  return gbcc_testing_gemm_ex2(M, N, K, A, B, Cout, slices, ksplit, bn_req, cta2, chunk, fold, 1, repeat, ms);
}

extern "C" int gbcc_testing_gemm_ex2(int64_t M, int64_t N, int64_t K, const double* A, const double* B,
                                     double* Cout, int slices, int ksplit, int bn_req, int cta2, int chunk,
                                     int fold, int sps, int repeat, float* ms) {
  return gbcc_testing_gemm_ex3(M, N, K, A, B, Cout, slices, ksplit, bn_req, cta2, chunk, fold, sps, 1, 0, repeat, ms);
}

extern "C" int gbcc_testing_gemm_ex3(int64_t M, int64_t N, int64_t K, const double* A, const double* B,
                                     double* Cout, int slices, int ksplit, int bn_req, int cta2, int chunk,
                                     int fold, int sps, int group, int cmode, int repeat, float* ms) {
  using namespace gbcc;
  const bool accumulate = (cmode & 1) != 0, m_major = (cmode & 2) != 0;
  if (M < 1 || N < 1 || K < 1 || !A || !B || !Cout || slices < 0 || slices > 3 || repeat < 1 || ksplit < 1 ||
      group < 0)
    return GBCC_ERR_INVALID_ARG;
  if (bn_req != 0 && bn_req != 32 && bn_req != 64 && bn_req != 128 && bn_req != 192 && bn_req != 256)
    return GBCC_ERR_INVALID_ARG;
  std::vector<void*> owned;
  auto alloc = [&](size_t bytes) {
    void* p = dev_alloc(bytes);
    owned.push_back(p);
    return p;
  };
  int status = GBCC_OK;
  try {
    cudaStream_t st = nullptr;
    double* dA = static_cast<double*>(alloc(M * K * sizeof(double)));
    double* dB = static_cast<double*>(alloc(N * K * sizeof(double)));
    double* dC = static_cast<double*>(alloc(M * N * sizeof(double)));
    int* err = static_cast<int*>(alloc(sizeof(int)));
    GBCC_CK(cudaMemset(err, 0, sizeof(int)));
    GBCC_CK(cudaMemcpy(dA, A, M * K * sizeof(double), cudaMemcpyDefault));
    GBCC_CK(cudaMemcpy(dB, B, N * K * sizeof(double), cudaMemcpyDefault));
    GBCC_CK(cudaMemset(dC, 0, M * N * sizeof(double)));
    auto table = [&](int64_t n, int64_t stride) {
      std::vector<int64_t> h(n);
      for (int64_t i = 0; i < n; ++i) h[i] = i * stride;
      int64_t* d = static_cast<int64_t*>(alloc(n * sizeof(int64_t)));
      GBCC_CK(cudaMemcpy(d, h.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice));
      return d;
    };
    // C row-major, or column-major (unit stride along M) with cmode bit 1
    const int64_t* cm = m_major ? table(M, 1) : table(M, N);
    const int64_t* cn = m_major ? table(N, M) : table(N, 1);
    const double beta = accumulate ? 1.0 : 0.0;
    cudaEvent_t e0, e1;
    GBCC_CK(cudaEventCreate(&e0));
    GBCC_CK(cudaEventCreate(&e1));
    if (slices == 0) {
      GemmF64Args g{};
      g.M = M; g.N = N; g.K = K;
      g.A = dA; g.lda = K; g.B = dB; g.ldb = K;
      g.C = dC; g.cm = cm; g.cn = cn; g.alpha = 1.0; g.beta = beta; g.m_major = m_major ? 1 : 0;
      if (ksplit > 1) {
        g.ksplit = ksplit;
        g.k_per_split = (K + ksplit - 1) / ksplit;
        g.ksplit = static_cast<int>((K + g.k_per_split - 1) / g.k_per_split);
        g.partial = static_cast<double*>(alloc(g.ksplit * M * N * sizeof(double)));
      }
      launch_gemm_f64(g, st);
      GBCC_CK(cudaEventRecord(e0, st));
      for (int r = 0; r < repeat; ++r) launch_gemm_f64(g, st);
      GBCC_CK(cudaEventRecord(e1, st));
      if (accumulate) {  // the output of one product added to zeros
        GBCC_CK(cudaMemsetAsync(dC, 0, M * N * sizeof(double), st));
        launch_gemm_f64(g, st);
      }
    } else {
      const int bn = bn_req ? bn_req : (cta2 ? (N <= 64 ? 64 : 128) : gemm_tc_pick_bn(N, false));
      const int64_t Mpad = rup(M, cta2 ? 2 * kTcBM : kTcBM), Npad = rup(N, bn), Kpad = rup(K, kTcBK);
      auto* sa = static_cast<__nv_bfloat16*>(alloc(slices * Mpad * Kpad * sizeof(__nv_bfloat16)));
      auto* sb = static_cast<__nv_bfloat16*>(alloc(slices * Npad * Kpad * sizeof(__nv_bfloat16)));
      auto pack = [&](const double* src, int64_t rows, int64_t rows_pad, __nv_bfloat16* dst) {
        GatherArgs g{};
        g.nterms = 1;
        g.t[0].coef = 1.0;
        g.t[0].a = src;
        g.t[0].ra = table(rows, K);
        g.t[0].ca = table(K, 1);
        g.R = rows; g.C = K; g.Rpad = rows_pad; g.Cpad = Kpad; g.ldo = Kpad;
        g.outs = dst; g.nslices = slices; g.slice_stride = rows_pad * Kpad;
        launch_gather(g, st);
      };
      pack(dA, M, Mpad, sa);
      pack(dB, N, Npad, sb);
      GemmTcArgs t{};
      t.M = M; t.N = N; t.Mpad = Mpad; t.Npad = Npad; t.Kpad = Kpad;
      t.A = sa; t.a_slices = slices; t.B = sb; t.b_slices = slices;
      for (int a = 0; a < slices; ++a)
        for (int b = 0; b < slices; ++b)
          if (a + b < slices) { t.pa[t.npairs] = a; t.pb[t.npairs] = b; ++t.npairs; }
      t.C = dC; t.cm = cm; t.cn = cn; t.alpha = 1.0; t.beta = beta; t.bn = bn; t.err = err;
      t.m_major = m_major ? 1 : 0;
      t.cta2 = cta2 ? 1 : 0;
      t.chunk = chunk;
      t.fold = fold;
      t.sps = sps;
      t.group = group;
      if (ksplit > 1) {
        const int64_t kblocks = Kpad / kTcBK;
        t.kb_per_split = static_cast<int>((kblocks + ksplit - 1) / ksplit);
        t.ksplit = static_cast<int>((kblocks + t.kb_per_split - 1) / t.kb_per_split);
        t.partial = static_cast<double*>(alloc(t.ksplit * Mpad * Npad * sizeof(double)));
      }
      auto run = [&]() {
        if (!launch_gemm_tc(t, st)) throw Error(GBCC_ERR_CUDA, "tcgen05 launch rejected");
        if (t.ksplit > 1)
          launch_splitk_reduce(M, N, t.ksplit, t.partial, Mpad, Npad, dC, cm, cn, 1.0, beta, st);
      };
      run();
      GBCC_CK(cudaEventRecord(e0, st));
      for (int r = 0; r < repeat; ++r) run();
      GBCC_CK(cudaEventRecord(e1, st));
      if (accumulate) {  // the output of one product added to zeros
        GBCC_CK(cudaMemsetAsync(dC, 0, M * N * sizeof(double), st));
        run();
      }
    }
    GBCC_CK(cudaEventSynchronize(e1));
    GBCC_CK(cudaGetLastError());
    float t_ms = 0.f;
    GBCC_CK(cudaEventElapsedTime(&t_ms, e0, e1));
    if (ms) *ms = t_ms / repeat;
    int herr = 0;
    GBCC_CK(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr != kDevOk) status = GBCC_ERR_TIMEOUT;
    if (m_major) {
      std::vector<double> cc(static_cast<size_t>(M * N));
      GBCC_CK(cudaMemcpy(cc.data(), dC, M * N * sizeof(double), cudaMemcpyDeviceToHost));
      for (int64_t m = 0; m < M; ++m)
        for (int64_t n = 0; n < N; ++n) Cout[m * N + n] = cc[n * M + m];
    } else {
      GBCC_CK(cudaMemcpy(Cout, dC, M * N * sizeof(double), cudaMemcpyDefault));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  } catch (const Error& e) {
    std::fprintf(stderr, "gbcc_testing_gemm: %s\n", e.what());
    status = e.status;
  }
  for (void* p : owned) dev_free(p);
  return status;
}

extern "C" int gbcc_testing_split(const double* x, int64_t n, int nslices, uint16_t* out) {
  using namespace gbcc;
  if (!x || !out || n < 0 || nslices < 1 || nslices > 3) return GBCC_ERR_INVALID_ARG;
  if (n == 0) return GBCC_OK;
  try {
    double* dx = static_cast<double*>(dev_alloc(n * sizeof(double)));
    unsigned short* dout = static_cast<unsigned short*>(dev_alloc(n * nslices * sizeof(unsigned short)));
    GBCC_CK(cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice));
    launch_split_test(dx, n, nslices, dout, nullptr);
    GBCC_CK(cudaGetLastError());
    GBCC_CK(cudaMemcpy(out, dout, n * nslices * sizeof(unsigned short), cudaMemcpyDeviceToHost));
    dev_free(dx);
    dev_free(dout);
    return GBCC_OK;
  } catch (const Error& e) {
    return e.status;
  }
}

extern "C" int gbcc_testing_scale(const double* x, int64_t n, double coef, double* out) {
  using namespace gbcc;
  if (!x || !out || n < 0) return GBCC_ERR_INVALID_ARG;
  if (n == 0) return GBCC_OK;
  try {
    double* dx = static_cast<double*>(dev_alloc(2 * n * sizeof(double)));
    GBCC_CK(cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice));
    launch_scale_test(dx, n, coef, dx + n, nullptr);
    GBCC_CK(cudaGetLastError());
    GBCC_CK(cudaMemcpy(out, dx + n, n * sizeof(double), cudaMemcpyDeviceToHost));
    dev_free(dx);
    return GBCC_OK;
  } catch (const Error& e) {
    return e.status;
  }
}

extern "C" int gbcc_testing_fp64_peak(double* gflops) {
  using namespace gbcc;
  if (!gflops) return GBCC_ERR_INVALID_ARG;
  try {
    int dev = 0, sms = 0;
    GBCC_CK(cudaGetDevice(&dev));
    GBCC_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = static_cast<double*>(dev_alloc(sizeof(double)));
    const int blocks = sms * 8, threads = 256, iters = 1 << 16;
    fp64_fma_probe<<<blocks, threads>>>(out, 1024);
    cudaEvent_t e0, e1;
    GBCC_CK(cudaEventCreate(&e0));
    GBCC_CK(cudaEventCreate(&e1));
    GBCC_CK(cudaEventRecord(e0));
    fp64_fma_probe<<<blocks, threads>>>(out, iters);
    GBCC_CK(cudaEventRecord(e1));
    GBCC_CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    GBCC_CK(cudaEventElapsedTime(&ms, e0, e1));
    dev_free(out);
    *gflops = 2.0 * 8.0 * iters * static_cast<double>(blocks) * threads / (ms * 1e-3) / 1e9;
    return GBCC_OK;
  } catch (const Error& e) {
    return e.status;
  }
}

extern "C" int gbcc_testing_dmma_peak(double* gflops) {
  using namespace gbcc;
  if (!gflops) return GBCC_ERR_INVALID_ARG;
  try {
    int dev = 0, sms = 0;
    GBCC_CK(cudaGetDevice(&dev));
    GBCC_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = static_cast<double*>(dev_alloc(sizeof(double)));
    const int blocks = sms * 4, threads = 256, iters = 1 << 14;
    fp64_dmma_probe<<<blocks, threads>>>(out, 256);
    cudaEvent_t e0, e1;
    GBCC_CK(cudaEventCreate(&e0));
    GBCC_CK(cudaEventCreate(&e1));
    GBCC_CK(cudaEventRecord(e0));
    fp64_dmma_probe<<<blocks, threads>>>(out, iters);
    GBCC_CK(cudaEventRecord(e1));
    GBCC_CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    GBCC_CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dev_free(out);
    const double warps = static_cast<double>(blocks) * threads / 32;
    *gflops = 512.0 * 4.0 * iters * warps / (ms * 1e-3) / 1e9;
    return GBCC_OK;
  } catch (const Error& e) {
    return e.status;
  }
}

namespace {

// Fixed-point pack of a row-major [rows][cols] FP64 matrix into the GEMM's
// slice panel ([nslices][Cpad/64][rows_pad][64]) through the gather kernels:
// row exponents zeroed, the exponent pass, the digit pass.
void fixed_pack(const double* src, int64_t rows, int64_t cols, int64_t rows_pad, int64_t cols_pad, int nslices,
                unsigned* rowexp, __nv_bfloat16* dst, const int64_t* ra, const int64_t* ca, cudaStream_t st) {
  using namespace gbcc;
  GatherArgs g{};
  g.nterms = 1;
  gather_set_coef(g.t[0], 1.0);
  g.t[0].a = src;
  g.t[0].ra = ra;
  g.t[0].ca = ca;
  g.plain = 1;
  g.R = rows; g.C = cols; g.Rpad = rows_pad; g.Cpad = cols_pad; g.ldo = cols_pad;
  g.outs = dst; g.nslices = nslices; g.slice_stride = rows_pad * cols_pad;
  g.rowexp = rowexp;
  GBCC_CK(cudaMemsetAsync(rowexp, 0, rows_pad * sizeof(unsigned), st));
  g.fixed = 1;
  launch_gather(g, st);
  g.fixed = 2;
  launch_gather(g, st);
}

}  // namespace

extern "C" int gbcc_testing_fixed_split(const double* x, int64_t rows, int64_t cols, int nslices, uint16_t* out,
                                        uint32_t* rowexp) {
  using namespace gbcc;
  if (!x || !out || !rowexp || rows < 1 || cols < 1 || nslices < 1 || nslices > kFixedSlices)
    return GBCC_ERR_INVALID_ARG;
  std::vector<void*> owned;
  auto alloc = [&](size_t bytes) {
    void* p = dev_alloc(bytes);
    owned.push_back(p);
    return p;
  };
  int status = GBCC_OK;
  try {
    const int64_t rows_pad = rup(rows, kTcBM), cols_pad = rup(cols, kTcBK);
    double* dx = static_cast<double*>(alloc(rows * cols * sizeof(double)));
    GBCC_CK(cudaMemcpy(dx, x, rows * cols * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<int64_t> hra(rows), hca(cols);
    for (int64_t r = 0; r < rows; ++r) hra[r] = r * cols;
    for (int64_t c = 0; c < cols; ++c) hca[c] = c;
    auto* ra = static_cast<int64_t*>(alloc(rows * sizeof(int64_t)));
    auto* ca = static_cast<int64_t*>(alloc(cols * sizeof(int64_t)));
    GBCC_CK(cudaMemcpy(ra, hra.data(), rows * sizeof(int64_t), cudaMemcpyHostToDevice));
    GBCC_CK(cudaMemcpy(ca, hca.data(), cols * sizeof(int64_t), cudaMemcpyHostToDevice));
    auto* re = static_cast<unsigned*>(alloc(rows_pad * sizeof(unsigned)));
    const int64_t n = nslices * rows_pad * cols_pad;
    auto* panel = static_cast<__nv_bfloat16*>(alloc(n * sizeof(__nv_bfloat16)));
    fixed_pack(dx, rows, cols, rows_pad, cols_pad, nslices, re, panel, ra, ca, nullptr);
    GBCC_CK(cudaGetLastError());
    std::vector<uint16_t> hp(n);
    GBCC_CK(cudaMemcpy(hp.data(), panel, n * sizeof(uint16_t), cudaMemcpyDeviceToHost));
    GBCC_CK(cudaMemcpy(rowexp, re, rows * sizeof(unsigned), cudaMemcpyDeviceToHost));
    // panel element (r, c) of slice s: s * rows_pad * cols_pad + (c / 64) * rows_pad * 64 + r * 64 + c % 64
    for (int s = 0; s < nslices; ++s)
      for (int64_t r = 0; r < rows; ++r)
        for (int64_t c = 0; c < cols; ++c)
          out[(s * rows + r) * cols + c] = hp[s * rows_pad * cols_pad + (c >> 6) * (rows_pad << 6) + (r << 6) + (c & 63)];
  } catch (const Error& e) {
    status = e.status;
  }
  for (void* p : owned) dev_free(p);
  return status;
}

extern "C" int gbcc_testing_gemm_fp64tc(int64_t M, int64_t N, int64_t K, const double* A, const double* B,
                                        double* Cout, int bn_req, int ksplit, int cta2, int repeat, float* ms) {
  using namespace gbcc;
  if (M < 1 || N < 1 || K < 1 || !A || !B || !Cout || repeat < 1 || ksplit < 1) return GBCC_ERR_INVALID_ARG;
  if (bn_req != 0 && bn_req != 32 && bn_req != 64 && bn_req != 128) return GBCC_ERR_INVALID_ARG;
  if (cta2 && bn_req != 64 && bn_req != 128) return GBCC_ERR_INVALID_ARG;
  std::vector<void*> owned;
  auto alloc = [&](size_t bytes) {
    void* p = dev_alloc(bytes);
    owned.push_back(p);
    return p;
  };
  int status = GBCC_OK;
  try {
    cudaStream_t st = nullptr;
    const int nsl = kFixedSlices;
    const int bn = bn_req ? bn_req : gemm_tc_pick_bn(N, false);
    const int64_t Mpad = rup(M, cta2 ? 2 * kTcBM : kTcBM), Npad = rup(N, bn), Kpad = rup(K, kTcBK);
    double* dA = static_cast<double*>(alloc(M * K * sizeof(double)));
    double* dB = static_cast<double*>(alloc(N * K * sizeof(double)));
    double* dC = static_cast<double*>(alloc(M * N * sizeof(double)));
    int* err = static_cast<int*>(alloc(sizeof(int)));
    GBCC_CK(cudaMemset(err, 0, sizeof(int)));
    GBCC_CK(cudaMemcpy(dA, A, M * K * sizeof(double), cudaMemcpyHostToDevice));
    GBCC_CK(cudaMemcpy(dB, B, N * K * sizeof(double), cudaMemcpyHostToDevice));
    auto table = [&](int64_t n, int64_t stride) {
      std::vector<int64_t> h(n);
      for (int64_t i = 0; i < n; ++i) h[i] = i * stride;
      int64_t* d = static_cast<int64_t*>(alloc(n * sizeof(int64_t)));
      GBCC_CK(cudaMemcpy(d, h.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice));
      return d;
    };
    const int64_t* cm = table(M, N);
    const int64_t* cn = table(N, 1);
    const int64_t* ck = table(K, 1);
    auto* sa = static_cast<__nv_bfloat16*>(alloc(nsl * Mpad * Kpad * sizeof(__nv_bfloat16)));
    auto* sb = static_cast<__nv_bfloat16*>(alloc(nsl * Npad * Kpad * sizeof(__nv_bfloat16)));
    auto* ea = static_cast<unsigned*>(alloc(Mpad * sizeof(unsigned)));
    auto* eb = static_cast<unsigned*>(alloc(Npad * sizeof(unsigned)));
    fixed_pack(dA, M, K, Mpad, Kpad, nsl, ea, sa, table(M, K), ck, st);
    fixed_pack(dB, N, K, Npad, Kpad, nsl, eb, sb, table(N, K), ck, st);
    GemmTcArgs t{};
    t.M = M; t.N = N; t.Mpad = Mpad; t.Npad = Npad; t.Kpad = Kpad;
    t.A = sa; t.a_slices = nsl; t.B = sb; t.b_slices = nsl;
    t.C = dC; t.cm = cm; t.cn = cn; t.alpha = 1.0; t.bn = bn; t.err = err;
    t.chunk = kFixedChunk;
    t.fold = kFixedFold;
    t.sps = 1;
    t.group = 1;
    t.cta2 = cta2 ? 1 : 0;
    if (ksplit > 1) {
      const int64_t kblocks = Kpad / kTcBK;
      t.kb_per_split = static_cast<int>((kblocks + ksplit - 1) / ksplit);
      t.ksplit = static_cast<int>((kblocks + t.kb_per_split - 1) / t.kb_per_split);
      t.partial = static_cast<double*>(alloc(t.ksplit * Mpad * Npad * sizeof(double)));
    }
    // one launch per weight class, smallest weight first, as the engine runs them
    auto run = [&]() {
      for (int w = nsl - 1; w >= 0; --w) {
        t.npairs = fixed_class_pairs(nsl, w, t.pa, t.pb);
        t.beta = w == nsl - 1 ? 0.0 : 1.0;
        if (!launch_gemm_tc(t, st)) throw Error(GBCC_ERR_CUDA, "tcgen05 launch rejected");
        if (t.ksplit > 1) launch_splitk_reduce(M, N, t.ksplit, t.partial, Mpad, Npad, dC, cm, cn, 1.0, t.beta, st);
      }
    };
    cudaEvent_t e0, e1;
    GBCC_CK(cudaEventCreate(&e0));
    GBCC_CK(cudaEventCreate(&e1));
    run();
    GBCC_CK(cudaEventRecord(e0, st));
    for (int r = 0; r < repeat; ++r) run();
    GBCC_CK(cudaEventRecord(e1, st));
    GBCC_CK(cudaEventSynchronize(e1));
    GBCC_CK(cudaGetLastError());
    float t_ms = 0.f;
    GBCC_CK(cudaEventElapsedTime(&t_ms, e0, e1));
    if (ms) *ms = t_ms / repeat;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int herr = 0;
    GBCC_CK(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr != kDevOk) status = GBCC_ERR_TIMEOUT;
    GBCC_CK(cudaMemcpy(Cout, dC, M * N * sizeof(double), cudaMemcpyDeviceToHost));
  } catch (const Error& e) {
    std::fprintf(stderr, "gbcc_testing_gemm_fp64tc: %s\n", e.what());
    status = e.status;
  }
  for (void* p : owned) dev_free(p);
  return status;
}

// Failure detection of the tensor-core pipeline: one GEMM whose producer
// leaves stage `skip_stage` of every CTA unloaded, with the barriers' wait
// limit shortened to wait_ns, so the MMA thread's bounded wait runs out; the
// kernel records the timeout, drains its copies, waits for its MMAs, frees
// TMEM and returns.  *first gets that launch's status (GBCC_ERR_TIMEOUT
// expected); the same product is then run normally and *second gets its
// status, C its result.
extern "C" int gbcc_testing_gemm_timeout(int64_t M, int64_t N, int64_t K, const double* A, const double* B,
                                         double* Cout, uint64_t wait_ns, int64_t skip_stage, int* first,
                                         int* second) {
  using namespace gbcc;
  if (M < 1 || N < 1 || K < 1 || !A || !B || !Cout || !first || !second || skip_stage < 0 || wait_ns == 0)
    return GBCC_ERR_INVALID_ARG;
  std::vector<void*> owned;
  auto alloc = [&](size_t bytes) {
    void* p = dev_alloc(bytes);
    owned.push_back(p);
    return p;
  };
  int status = GBCC_OK;
  try {
    cudaStream_t st = nullptr;
    const int slices = 3, bn = 128;
    const int64_t Mpad = rup(M, kTcBM), Npad = rup(N, bn), Kpad = rup(K, kTcBK);
    double* dA = static_cast<double*>(alloc(M * K * sizeof(double)));
    double* dB = static_cast<double*>(alloc(N * K * sizeof(double)));
    double* dC = static_cast<double*>(alloc(M * N * sizeof(double)));
    int* err = static_cast<int*>(alloc(sizeof(int)));
    GBCC_CK(cudaMemcpy(dA, A, M * K * sizeof(double), cudaMemcpyHostToDevice));
    GBCC_CK(cudaMemcpy(dB, B, N * K * sizeof(double), cudaMemcpyHostToDevice));
    auto table = [&](int64_t n, int64_t stride) {
      std::vector<int64_t> h(n);
      for (int64_t i = 0; i < n; ++i) h[i] = i * stride;
      int64_t* d = static_cast<int64_t*>(alloc(n * sizeof(int64_t)));
      GBCC_CK(cudaMemcpy(d, h.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice));
      return d;
    };
    auto* sa = static_cast<__nv_bfloat16*>(alloc(slices * Mpad * Kpad * sizeof(__nv_bfloat16)));
    auto* sb = static_cast<__nv_bfloat16*>(alloc(slices * Npad * Kpad * sizeof(__nv_bfloat16)));
    auto pack = [&](const double* src, int64_t rows, int64_t rows_pad, __nv_bfloat16* dst) {
      GatherArgs g{};
      g.nterms = 1;
      gather_set_coef(g.t[0], 1.0);
      g.t[0].a = src;
      g.t[0].ra = table(rows, K);
      g.t[0].ca = table(K, 1);
      g.plain = 1;
      g.R = rows; g.C = K; g.Rpad = rows_pad; g.Cpad = Kpad; g.ldo = Kpad;
      g.outs = dst; g.nslices = slices; g.slice_stride = rows_pad * Kpad;
      launch_gather(g, st);
    };
    pack(dA, M, Mpad, sa);
    pack(dB, N, Npad, sb);
    GemmTcArgs t{};
    t.M = M; t.N = N; t.Mpad = Mpad; t.Npad = Npad; t.Kpad = Kpad;
    t.A = sa; t.a_slices = slices; t.B = sb; t.b_slices = slices;
    for (int a = 0; a < slices; ++a)
      for (int b = 0; b < slices; ++b)
        if (a + b < slices) { t.pa[t.npairs] = a; t.pb[t.npairs] = b; ++t.npairs; }
    t.C = dC; t.cm = table(M, N); t.cn = table(N, 1); t.alpha = 1.0; t.beta = 0.0; t.bn = bn; t.err = err;
    t.chunk = 4; t.sps = 1; t.group = 1;
    auto run = [&](int64_t skip1, uint64_t limit) {
      GBCC_CK(cudaMemset(err, 0, sizeof(int)));
      t.skip_stage1 = skip1;
      t.wait_ns = limit;
      if (!launch_gemm_tc(t, st)) throw Error(GBCC_ERR_CUDA, "tcgen05 launch rejected");
      GBCC_CK(cudaStreamSynchronize(st));
      GBCC_CK(cudaGetLastError());
      int herr = 0;
      GBCC_CK(cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost));
      return herr == kDevOk ? static_cast<int>(GBCC_OK) : static_cast<int>(GBCC_ERR_TIMEOUT);
    };
    *first = run(skip_stage + 1, wait_ns);
    *second = run(0, 0);
    GBCC_CK(cudaMemcpy(Cout, dC, M * N * sizeof(double), cudaMemcpyDeviceToHost));
  } catch (const Error& e) {
    std::fprintf(stderr, "gbcc_testing_gemm_timeout: %s\n", e.what());
    status = e.status;
  }
  for (void* p : owned) dev_free(p);
  return status;
}

// The DIIS coefficient solve of the solver (diis_coefficients) on a given B:
// host arrays in and out, its own stream.
extern "C" int gbcc_testing_diis_coefficients(int32_t n, const double* B, double damping, double* coef,
                                              int32_t* nskip) {
  if (n < 1 || n > 16 || !B || !coef || !nskip) return GBCC_ERR_INVALID_ARG;
  double *dB = nullptr, *dc = nullptr;
  int* dn = nullptr;
  cudaStream_t st = nullptr;
  int status = GBCC_OK;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&dB, sizeof(double) * n * n) != cudaSuccess || cudaMalloc(&dc, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&dn, sizeof(int)) != cudaSuccess ||
      cudaMemcpyAsync(dB, B, sizeof(double) * n * n, cudaMemcpyHostToDevice, st) != cudaSuccess) {
    status = GBCC_ERR_CUDA;
  } else {
    gbcc::launch_diis_coefficients_test(dB, n, damping, dc, dn, st);
    int h_n = 0;
    if (cudaMemcpyAsync(coef, dc, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&h_n, dn, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      status = GBCC_ERR_CUDA;
    *nskip = h_n;
  }
  cudaGetLastError();
  cudaFree(dB);
  cudaFree(dc);
  cudaFree(dn);
  if (st) cudaStreamDestroy(st);
  return status;
}
