// Perturbative triples correction (T) of closed-shell CCSD on the GPU.
//
// The reference's "straight" (T) (src/mpqc/chemistry/qc/lcao/cc/ccsd_t.h:
// 1127-1167, denominators by CCSD_T_Reduce, :2274-2333) forms the connected
// triples of all occupied triplets at once (o^3 v^3 elements).  Here the
// triplets run in batches: for each pair i <= j, the triplets (i, j, k) with
// k >= j (a triplet's abc sum is the same for every ordering of i, j, k, so it
// counts once per distinct ordering).  A batch's
//   W[k][a][b][c] = t3(a,b,c,i,j,k) = sum over the six simultaneous
//   permutations of (a,i),(b,j),(c,k) of
//     X(a,b,c,i,j,k) = sum_d <id|ab> t2(d,c,j,k) - sum_l <jk|lc> t2(a,b,i,l)
// is six GEMMs, one per permutation term, each over K = v + o (the d and l
// sums concatenated along K), whose outputs are scattered into W through the
// term's offset tables: each term keeps one of its operands fixed over the
// batch and stacks the other over k, so every GEMM covers the whole batch,
// and each writes along W's unit stride (c) in its epilogue's lane
// direction.  The energy kernel then reads W at the six
// virtual-index permutations that stand for t3's occupied-index permutations
// (t3(abc,kij) = W[b][c][a], ...), adds the disconnected v3 from <ij|ab> and
// t1, and divides by e_i + e_j + e_k - e_a - e_b - e_c.
//
// Operand panels (rows x K, K = v + o contiguous: columns d < v, then l),
// packed once:
//   A  [(x,p,q)] = ( <xd|pq> = Giabc[x][d][p][q] , -t2(p,q,x,l) )
//   At [(x,q,p)] = the same rows with p fastest
//   B  [(y,z,c)] = ( t2(d,c,y,z) , <yz|lc> = Gijka[y][z][l][c] )
//   B2 [(y,z,b)] = ( t2(b,d,y,z) = t2(d,b,z,y) , <zy|lb> = Gijka[z][y][l][b] )
// in FP64 (precision FP64: the DFMA GEMM), three BF16 slices (MIXED) or six
// fixed-point slices (FP64_TC, one launch per weight class).
#include <algorithm>
#include <deque>
#include <vector>

#include "../../include/gbcc.h"
#include "engine.h"
#include "kernels.h"
#include "triples.h"

namespace gbcc {

// test hook: triplets per batch (0: as many as keep the t3 slice in L2)
int64_t g_triples_chunk = 0;

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double block_sum_det(double v, double* sh) {
  // fixed-order tree reduction (deterministic)
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

// One batch (i, j; k = k0 + kk): block (a, kk) sums over (b, c) and writes the
// weighted partial to partial[kk * v + a].  R: the arithmetic of the terms
// (double for the FP64-grade precisions; float for MIXED, whose contractions
// already carry ~1e-6 relative error), summed per thread in FP64.
template <typename R>
__global__ void __launch_bounds__(kThreads) triples_energy_kernel(
    const double* __restrict__ W, int64_t o, int64_t v, int i, int j, int k0, int nk, const double* __restrict__ Gijab,
    const double* __restrict__ t1, const double* __restrict__ eps_o, const double* __restrict__ eps_v,
    double* __restrict__ partial) {
  __shared__ double sh[kThreads];
  const int64_t a = blockIdx.x;
  const int kk = blockIdx.y;
  const int k = k0 + kk;
  if (kk >= nk) return;
  const double mult = (i < j && j < k) ? 6.0 : ((i == j && j == k) ? 1.0 : 3.0);
  const int64_t v2 = v * v;
  const double* __restrict__ Wk = W + static_cast<int64_t>(kk) * v2 * v;
  const R base = static_cast<R>(eps_o[i] + eps_o[j] + eps_o[k] - eps_v[a]);
  const R t1ai = static_cast<R>(t1[a * o + i]);
  const double* __restrict__ g_ij = Gijab + (static_cast<int64_t>(i) * o + j) * v2;  // <ij|..>
  const double* __restrict__ g_jk = Gijab + (static_cast<int64_t>(j) * o + k) * v2;
  const double* __restrict__ g_ik = Gijab + (static_cast<int64_t>(i) * o + k) * v2;
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < v2; e += blockDim.x) {
    const int64_t b = e / v, c = e - b * v;
    const R w = static_cast<R>(Wk[a * v2 + b * v + c]);
    const R y = R(4) * w + static_cast<R>(Wk[b * v2 + c * v + a]) + static_cast<R>(Wk[c * v2 + a * v + b]) -
                R(2) * (static_cast<R>(Wk[c * v2 + b * v + a]) + static_cast<R>(Wk[a * v2 + c * v + b]) +
                        static_cast<R>(Wk[b * v2 + a * v + c]));
    const R vv = static_cast<R>(g_ij[a * v + b]) * static_cast<R>(t1[c * o + k]) +
                 static_cast<R>(g_jk[b * v + c]) * t1ai +
                 static_cast<R>(g_ik[a * v + c]) * static_cast<R>(t1[b * o + j]);
    const R d = base - static_cast<R>(eps_v[b]) - static_cast<R>(eps_v[c]);
    acc += static_cast<double>((w + vv) * y / d);
  }
  const double s = block_sum_det(acc, sh);
  if (threadIdx.x == 0) partial[static_cast<int64_t>(kk) * v + a] = mult * s;
}

__global__ void __launch_bounds__(kThreads) sum_kernel(const double* __restrict__ x, int64_t n, double scale,
                                                      double* __restrict__ out) {
  __shared__ double sh[kThreads];
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) acc += x[e];
  const double s = block_sum_det(acc, sh);
  if (threadIdx.x == 0) *out = scale * s;
}

int64_t rup(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// A packed operand: rows x K, FP64 rows (precision FP64) or a slice panel.
struct Panel {
  int64_t rows = 0, K = 0, rows_pad = 0, Kpad = 0;
  double* f64 = nullptr;
  __nv_bfloat16* bf = nullptr;
  unsigned* rowexp = nullptr;
};

class Triples {
 public:
  Triples(const TriplesInputs& in, int precision, cudaStream_t st, int* err)
      : in_(in), prec_(precision), st_(st), err_(err) {
    slices_ = precision == GBCC_PREC_MIXED ? 3 : (precision == GBCC_PREC_FP64_TC ? kFixedSlices : 0);
  }
  ~Triples() {
    for (void* p : owned_) dev_free(p);
  }

  double run();

 private:
  void* alloc(size_t bytes) {
    void* p = dev_alloc(bytes);
    owned_.push_back(p);
    return p;
  }
  const int64_t* table(const std::vector<int64_t>& h) {
    auto* d = static_cast<int64_t*>(alloc(std::max<size_t>(h.size(), 1) * sizeof(int64_t)));
    tables_.push_back(h);  // the copy's source lives until run() returns
    const std::vector<int64_t>& src = tables_.back();
    if (!src.empty())
      GBCC_CK(cudaMemcpyAsync(d, src.data(), src.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st_));
    return d;
  }
  Panel pack(const double* src1, int64_t n1, const std::vector<int64_t>& ra1, const std::vector<int64_t>& ca1,
             double coef1, const double* src2, int64_t n2, const std::vector<int64_t>& ra2,
             const std::vector<int64_t>& ca2, double coef2, int64_t split);
  void gemm(const Panel& A, int64_t a0, int64_t M, const Panel& B, int64_t b0, int64_t N, const int64_t* cm,
            const int64_t* cn, bool m_major, double beta);

  TriplesInputs in_;
  int prec_, slices_ = 0;
  cudaStream_t st_;
  int* err_;
  std::vector<void*> owned_;
  std::deque<std::vector<int64_t>> tables_;  // stable addresses
  double* partk_ = nullptr;  // K-split partial tiles
  size_t partk_elems_ = 0;
  double* W_ = nullptr;      // t3 of one batch, [k - j][a][b][c]
  double* mask_ = nullptr;   // {0.0, 1.0}
};

// A panel whose columns c < v come from src1 and the rest from src2 (the d
// and l sums side by side): two gather terms, each multiplied by a 0/1 mask
// over the columns (a 2-element table), so every column takes one source.
// The offsets of both terms are checked against their sources on the host.
Panel Triples::pack(const double* src1, int64_t n1, const std::vector<int64_t>& ra1, const std::vector<int64_t>& ca1,
                    double coef1, const double* src2, int64_t n2, const std::vector<int64_t>& ra2,
                    const std::vector<int64_t>& ca2, double coef2, int64_t split) {
  const int64_t rows = static_cast<int64_t>(ra1.size()), K = static_cast<int64_t>(ca1.size());
  auto inside = [](const std::vector<int64_t>& r, const std::vector<int64_t>& c, int64_t n) {
    const int64_t lo = *std::min_element(r.begin(), r.end()) + *std::min_element(c.begin(), c.end());
    const int64_t hi = *std::max_element(r.begin(), r.end()) + *std::max_element(c.begin(), c.end());
    return lo >= 0 && hi < n;
  };
  if (static_cast<int64_t>(ra2.size()) != rows || static_cast<int64_t>(ca2.size()) != K || !inside(ra1, ca1, n1) ||
      !inside(ra2, ca2, n2) || split < 0 || split > K)
    throw Error(GBCC_ERR_STATE, "(T): operand offsets outside the source");
  Panel p;
  p.rows = rows;
  p.K = K;
  std::vector<int64_t> zero(static_cast<size_t>(rows), 0), m1(static_cast<size_t>(K)), m2(static_cast<size_t>(K));
  for (int64_t c = 0; c < K; ++c) {
    m1[c] = c < split ? 1 : 0;  // index into mask_ = {0.0, 1.0}
    m2[c] = c < split ? 0 : 1;
  }
  const int64_t* rz = table(zero);
  GatherArgs g{};
  g.nterms = 2;
  g.products = 1;
  gather_set_coef(g.t[0], coef1);
  g.t[0].a = src1;
  g.t[0].ra = table(ra1);
  g.t[0].ca = table(ca1);
  g.t[0].b = mask_;
  g.t[0].rb = rz;
  g.t[0].cb = table(m1);
  gather_set_coef(g.t[1], coef2);
  g.t[1].a = src2;
  g.t[1].ra = table(ra2);
  g.t[1].ca = table(ca2);
  g.t[1].b = mask_;
  g.t[1].rb = rz;
  g.t[1].cb = table(m2);
  gather_finish(g);
  g.R = rows;
  g.C = K;
  if (slices_ == 0) {
    p.rows_pad = rows;
    p.Kpad = K;
    p.f64 = static_cast<double*>(alloc(static_cast<size_t>(rows) * K * sizeof(double)));
    g.Rpad = rows;
    g.Cpad = K;
    g.ldo = K;
    g.out = p.f64;
    launch_gather(g, st_);
    return p;
  }
  // rows padded for the widest tile (256): a window's tiles past the last
  // row fall outside the tensor map and load as zeros
  p.rows_pad = rup(rows, 256);
  p.Kpad = rup(K, kTcBK);
  p.bf = static_cast<__nv_bfloat16*>(alloc(static_cast<size_t>(slices_) * p.rows_pad * p.Kpad * sizeof(__nv_bfloat16)));
  g.Rpad = p.rows_pad;
  g.Cpad = p.Kpad;
  g.ldo = p.Kpad;
  g.outs = p.bf;
  g.nslices = slices_;
  g.slice_stride = p.rows_pad * p.Kpad;
  if (prec_ == GBCC_PREC_FP64_TC) {
    p.rowexp = static_cast<unsigned*>(alloc(static_cast<size_t>(p.rows_pad) * sizeof(unsigned)));
    GBCC_CK(cudaMemsetAsync(p.rowexp, 0, static_cast<size_t>(p.rows_pad) * sizeof(unsigned), st_));
    g.rowexp = p.rowexp;
    g.fixed = 1;
    launch_gather(g, st_);
    g.fixed = 2;
  }
  launch_gather(g, st_);
  return p;
}

// C[cm[m] + cn[n]] = beta C + alpha sum_k A[a0 + m][k] B[b0 + n][k], m < M, n < N
void Triples::gemm(const Panel& A, int64_t a0, int64_t M, const Panel& B, int64_t b0, int64_t N, const int64_t* cm,
                   const int64_t* cn, bool m_major, double beta) {
  const double alpha = 1.0;
  if (M <= 0 || N <= 0) return;
  // the operand windows lie inside their panels (checked on the host)
  if (a0 < 0 || a0 + M > A.rows || b0 < 0 || b0 + N > B.rows || A.K != B.K)
    throw Error(GBCC_ERR_STATE, "(T): GEMM window outside its operand panel");
  if (slices_ == 0) {
    GemmF64Args f{};
    f.M = M;
    f.N = N;
    f.K = A.K;
    f.A = A.f64 + a0 * A.K;
    f.lda = A.K;
    f.B = B.f64 + b0 * B.K;
    f.ldb = B.K;
    f.C = W_;
    f.cm = cm;
    f.cn = cn;
    f.alpha = alpha;
    f.beta = beta;
    f.m_major = m_major ? 1 : 0;
    launch_gemm_f64(f, st_);
    return;
  }
  const bool emu = prec_ == GBCC_PREC_FP64_TC;
  GemmTcArgs t{};
  t.M = M;
  t.N = N;
  t.bn = gemm_tc_pick_bn(N, !emu);
  t.Mpad = rup(M, kTcBM);
  t.Npad = rup(N, t.bn);
  t.Kpad = A.Kpad;
  t.A = A.bf;
  t.a_slices = slices_;
  t.a_rows = A.rows_pad;
  t.a_row0 = a0;
  t.B = B.bf;
  t.b_slices = slices_;
  t.b_rows = B.rows_pad;
  t.b_row0 = b0;
  t.C = W_;
  t.cm = cm;
  t.cn = cn;
  t.alpha = alpha;
  t.m_major = m_major ? 1 : 0;
  t.err = err_;
  t.sps = 1;
  t.group = 1;
  t.chunk = emu ? kFixedChunk : 4;
  t.fold = emu ? kFixedFold : 0;
  // fewer output tiles than SMs (the last batches): split K over CTAs
  const int64_t tiles = (t.Mpad / kTcBM) * (t.Npad / t.bn), kblocks = t.Kpad / kTcBK;
  const int64_t sms = num_sms();
  if (tiles < sms && kblocks >= 4) {
    int64_t ks = std::min<int64_t>((sms + tiles - 1) / tiles, kblocks / 2);
    if (ks > 1) {
      const int64_t kbps = (kblocks + ks - 1) / ks;
      ks = (kblocks + kbps - 1) / kbps;
      const size_t need = static_cast<size_t>(ks) * t.Mpad * t.Npad;
      if (need > partk_elems_) throw Error(GBCC_ERR_STATE, "(T): K-split workspace too small");
      t.ksplit = static_cast<int>(ks);
      t.kb_per_split = static_cast<int>(kbps);
      t.partial = partk_;
    }
  }
  auto launch = [&](double b) {
    t.beta = b;
    if (!launch_gemm_tc(t, st_)) throw Error(GBCC_ERR_CUDA, "(T): tcgen05 GEMM launch rejected");
    if (t.ksplit > 1)
      launch_splitk_reduce(M, N, t.ksplit, partk_, t.Mpad, t.Npad, W_, cm, cn, alpha, b, st_);
  };
  if (!emu) {
    t.npairs = 0;
    for (int p = 0; p < slices_; ++p)
      for (int q = 0; q < slices_; ++q)
        if (p + q < slices_) {
          t.pa[t.npairs] = p;
          t.pb[t.npairs] = q;
          ++t.npairs;
        }
    launch(beta);
    return;
  }
  for (int w = slices_ - 1; w >= 0; --w) {
    t.npairs = fixed_class_pairs(slices_, w, t.pa, t.pb);
    launch(w == slices_ - 1 ? beta : 1.0);
  }
}

double Triples::run() {
  const int64_t o = in_.o, v = in_.v, v2 = v * v, v3 = v2 * v, o2 = o * o, K = v + o;
  const int64_t nG = o * v3, nT = v2 * o2, nR = o2 * o * v;
  mask_ = static_cast<double*>(alloc(2 * sizeof(double)));
  {
    static const double m[2] = {0.0, 1.0};
    GBCC_CK(cudaMemcpyAsync(mask_, m, sizeof(m), cudaMemcpyHostToDevice, st_));
  }
  // ---- operand panels, columns (d < v | l)
  std::vector<int64_t> ra1, ra2, ca1(static_cast<size_t>(K)), ca2(static_cast<size_t>(K));
  auto cols = [&](int64_t sd, int64_t sl) {  // column offsets of the two sources (0 where masked)
    for (int64_t c = 0; c < K; ++c) {
      ca1[c] = c < v ? c * sd : 0;
      ca2[c] = c < v ? 0 : (c - v) * sl;
    }
  };
  // A[(x,p,q)] = (Giabc[x][d][p][q], -t2[p][q][x][l]); At: rows (x,q,p)
  ra1.assign(static_cast<size_t>(o * v2), 0);
  ra2.assign(static_cast<size_t>(o * v2), 0);
  for (int64_t x = 0; x < o; ++x)
    for (int64_t p = 0; p < v; ++p)
      for (int64_t q = 0; q < v; ++q) {
        ra1[(x * v + p) * v + q] = x * v3 + p * v + q;
        ra2[(x * v + p) * v + q] = p * v * o2 + q * o2 + x * o;
      }
  cols(v2, 1);
  const Panel A = pack(in_.Giabc, nG, ra1, ca1, 1.0, in_.t2, nT, ra2, ca2, -1.0, v);
  for (int64_t x = 0; x < o; ++x)
    for (int64_t q = 0; q < v; ++q)
      for (int64_t p = 0; p < v; ++p) {
        ra1[(x * v + q) * v + p] = x * v3 + p * v + q;
        ra2[(x * v + q) * v + p] = p * v * o2 + q * o2 + x * o;
      }
  const Panel At = pack(in_.Giabc, nG, ra1, ca1, 1.0, in_.t2, nT, ra2, ca2, -1.0, v);
  // B[(y,z,c)] = (t2[d][c][y][z], Gijka[y][z][l][c]); B2[(y,z,b)] = (t2[b][d][y][z], Gijka[z][y][l][b])
  ra1.assign(static_cast<size_t>(o2 * v), 0);
  ra2.assign(static_cast<size_t>(o2 * v), 0);
  for (int64_t y = 0; y < o; ++y)
    for (int64_t z = 0; z < o; ++z)
      for (int64_t c = 0; c < v; ++c) {
        ra1[(y * o + z) * v + c] = c * o2 + y * o + z;
        ra2[(y * o + z) * v + c] = (y * o + z) * o * v + c;
      }
  cols(v * o2, v);
  const Panel B = pack(in_.t2, nT, ra1, ca1, 1.0, in_.Gijka, nR, ra2, ca2, 1.0, v);
  for (int64_t y = 0; y < o; ++y)
    for (int64_t z = 0; z < o; ++z)
      for (int64_t b = 0; b < v; ++b) {
        ra1[(y * o + z) * v + b] = b * v * o2 + y * o + z;
        ra2[(y * o + z) * v + b] = (z * o + y) * o * v + b;
      }
  cols(o2, v);
  const Panel B2 = pack(in_.t2, nT, ra1, ca1, 1.0, in_.Gijka, nR, ra2, ca2, 1.0, v);

  // ---- output offset tables of the six permutation terms into W[kk][a][b][c]
  std::vector<int64_t> h;
  auto pq_table = [&](int64_t sp, int64_t sq) {  // rows (p, q): p sp + q sq
    h.assign(static_cast<size_t>(v2), 0);
    for (int64_t p = 0; p < v; ++p)
      for (int64_t q = 0; q < v; ++q) h[p * v + q] = p * sp + q * sq;
    return table(h);
  };
  auto kr_table = [&](int64_t sr) {  // rows (kk, r): kk v^3 + r sr
    h.assign(static_cast<size_t>(o * v), 0);
    for (int64_t kk = 0; kk < o; ++kk)
      for (int64_t r = 0; r < v; ++r) h[kk * v + r] = kk * v3 + r * sr;
    return table(h);
  };
  auto kqp_table = [&](int64_t sq, int64_t sp) {  // rows (kk, q, p): kk v^3 + q sq + p sp
    h.assign(static_cast<size_t>(o * v2), 0);
    for (int64_t kk = 0; kk < o; ++kk)
      for (int64_t q = 0; q < v; ++q)
        for (int64_t p = 0; p < v; ++p) h[(kk * v + q) * v + p] = kk * v3 + q * sq + p * sp;
    return table(h);
  };
  auto r_table = [&](int64_t sr) {
    h.assign(static_cast<size_t>(v), 0);
    for (int64_t r = 0; r < v; ++r) h[r] = r * sr;
    return table(h);
  };
  // term 1 (a,b,c,i,j,k): rows (a,b) x (kk,c), lanes along N (c)
  // term 2 (a,c,b,i,k,j): rows (a,c) x (kk,b), lanes along M (c)
  // term 3 (b,a,c,j,i,k): rows (b,a) x (kk,c), lanes along N
  // term 4 (b,c,a,j,k,i): rows (b,c) x (kk,a), lanes along M
  // term 5 (c,a,b,k,i,j): rows (kk,a,c) of At x b, lanes along M
  // term 6 (c,b,a,k,j,i): rows (kk,b,c) of At x a, lanes along M
  const int64_t* cm1 = pq_table(v2, v);
  const int64_t* cm2 = pq_table(v2, 1);
  const int64_t* cm3 = pq_table(v, v2);
  const int64_t* cm4 = pq_table(v, 1);
  const int64_t* cn13 = kr_table(1);
  const int64_t* cn2 = kr_table(v);
  const int64_t* cn4 = kr_table(v2);
  const int64_t* cm5 = kqp_table(v2, 1);
  const int64_t* cm6 = kqp_table(v, 1);
  const int64_t* cn5 = r_table(v);
  const int64_t* cn6 = r_table(v2);

  // K-split workspace: a split happens only with fewer output tiles than
  // SMs, ks <= ceil(SMs / tiles), so ks Mpad Npad < 2 SMs x one 128 x 256 tile
  if (slices_ > 0) {
    partk_elems_ = static_cast<size_t>(num_sms()) * 2 * kTcBM * 256;
    partk_ = static_cast<double*>(alloc(partk_elems_ * sizeof(double)));
  }
  // triplets per batch: all k >= j, unless their slice of t3 would pass
  // 8 GB (then chunks of k).  Chunks small enough to keep the slice in L2
  // measured slower (the batches' GEMMs shrink and multiply: (H2O)10 mixed
  // 18 s -> 28 s), so chunking only bounds memory.
  int64_t kc = std::max<int64_t>(1, std::min<int64_t>(o, (static_cast<int64_t>(8) << 30) / (v3 * 8)));
  if (g_triples_chunk > 0) kc = std::min<int64_t>(o, g_triples_chunk);
  {
    // largest offset each term writes, for the largest batch (kk < kc)
    const int64_t last = v - 1, kmax = kc - 1;
    const int64_t worst[] = {last * (v2 + v) + kmax * v3 + last,       // 1, 3
                             last * (v2 + 1) + kmax * v3 + last * v,   // 2
                             last * (v + 1) + kmax * v3 + last * v2,   // 4
                             kmax * v3 + last * (v2 + 1) + last * v,   // 5
                             kmax * v3 + last * (v + 1) + last * v2};  // 6
    for (int64_t w : worst)
      if (w >= kc * v3) throw Error(GBCC_ERR_STATE, "(T): output offsets outside W");
  }
  W_ = static_cast<double*>(alloc(static_cast<size_t>(kc) * v3 * sizeof(double)));
  const int64_t npair = o * (o + 1) / 2;
  double* partial = static_cast<double*>(alloc(static_cast<size_t>(npair) * o * v * sizeof(double)));
  GBCC_CK(cudaMemsetAsync(partial, 0, static_cast<size_t>(npair) * o * v * sizeof(double), st_));
  double* d_e = static_cast<double*>(alloc(sizeof(double)));

  int64_t slot = 0;
  for (int i = 0; i < o; ++i) {
    for (int j = i; j < o; ++j, ++slot) {
      const int64_t pij = (static_cast<int64_t>(i) * o + j) * v;  // rows (i, j, r)
      for (int k0 = j; k0 < o; k0 += static_cast<int>(kc)) {
        const int nk = static_cast<int>(std::min<int64_t>(kc, o - k0));
        const int64_t rj = (static_cast<int64_t>(j) * o + k0) * v;  // rows (j, k = k0.., r)
        const int64_t ri = (static_cast<int64_t>(i) * o + k0) * v;  // rows (i, k = k0.., r)
        const int64_t nkv = static_cast<int64_t>(nk) * v;
        gemm(A, i * v2, v2, B, rj, nkv, cm1, cn13, false, 0.0);
        gemm(A, i * v2, v2, B2, rj, nkv, cm2, cn2, true, 1.0);
        gemm(A, j * v2, v2, B, ri, nkv, cm3, cn13, false, 1.0);
        gemm(A, j * v2, v2, B2, ri, nkv, cm4, cn4, true, 1.0);
        gemm(At, static_cast<int64_t>(k0) * v2, nk * v2, B, pij, v, cm5, cn5, true, 1.0);
        gemm(At, static_cast<int64_t>(k0) * v2, nk * v2, B2, pij, v, cm6, cn6, true, 1.0);
        const dim3 grid(static_cast<unsigned>(v), static_cast<unsigned>(nk));
        double* part = partial + slot * o * v + static_cast<int64_t>(k0 - j) * v;
        if (prec_ == GBCC_PREC_MIXED)
          triples_energy_kernel<float><<<grid, kThreads, 0, st_>>>(W_, o, v, i, j, k0, nk, in_.Gijab, in_.t1,
                                                                    in_.eps_o, in_.eps_v, part);
        else
          triples_energy_kernel<double><<<grid, kThreads, 0, st_>>>(W_, o, v, i, j, k0, nk, in_.Gijab, in_.t1,
                                                                     in_.eps_o, in_.eps_v, part);
      }
    }
  }
  sum_kernel<<<1, kThreads, 0, st_>>>(partial, npair * o * v, 1.0 / 3.0, d_e);
  double e = 0.0;
  GBCC_CK(cudaMemcpyAsync(&e, d_e, sizeof(double), cudaMemcpyDeviceToHost, st_));
  GBCC_CK(cudaStreamSynchronize(st_));
  GBCC_CK(cudaGetLastError());
  return e;
}

}  // namespace

double triples_energy(const TriplesInputs& in, int precision, cudaStream_t st, int* err) {
  Triples t(in, precision, st, err);
  return t.run();
}

}  // namespace gbcc

extern "C" int gbcc_testing_triples_chunk(int64_t k) {
  if (k < 0) return GBCC_ERR_INVALID_ARG;
  gbcc::g_triples_chunk = k;
  return GBCC_OK;
}
