// Contraction planner and executor (see engine.h).
#include "engine.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

namespace gbcc {

// Autotune choices shared by every handle of the process, by contraction
// shape: a handle whose contractions were timed before (by another handle, or
// in an earlier process whose table was saved and loaded) takes the stored
// tile instead of timing its candidates again.
namespace {
struct TuneChoice {
  int bn, ksplit, sps, group;
  int64_t kps;
};
std::mutex g_tune_mu;
std::map<std::string, TuneChoice>& tune_table() {
  static std::map<std::string, TuneChoice> t;
  return t;
}
}  // namespace

bool tune_save(const std::string& path) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::ofstream f(path);
  if (!f) return false;
  f << "gbcc-autotune 1\n";
  for (const auto& kv : tune_table())
    f << kv.first << ' ' << kv.second.bn << ' ' << kv.second.ksplit << ' ' << kv.second.kps << ' '
      << kv.second.sps << ' ' << kv.second.group << '\n';
  return static_cast<bool>(f);
}

bool tune_load(const std::string& path) {
  std::ifstream f(path);
  if (!f) return false;
  std::string line;
  if (!std::getline(f, line) || line != "gbcc-autotune 1") return false;
  std::map<std::string, TuneChoice> add;
  while (std::getline(f, line)) {
    if (line.empty()) continue;
    std::istringstream is(line);
    std::string key;
    TuneChoice c{};
    if (!(is >> key >> c.bn >> c.ksplit >> c.kps >> c.sps >> c.group)) return false;
    std::string extra;
    if (is >> extra) return false;
    if (c.bn <= 0 || c.bn > 256 || c.ksplit < 1 || c.kps < 0 || c.sps < 1 || c.sps > 2 || c.group < 1) return false;
    add[key] = c;
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (const auto& kv : add) tune_table()[kv.first] = kv.second;
  return true;
}

void tune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_table().clear();
}

// test hooks (gbcc_testing_fail_alloc): device allocations made so far, and
// how many more succeed before one fails as if the device were full (-1: all)
std::atomic<int64_t> g_alloc_count{0};
std::atomic<int64_t> g_fail_alloc_after{-1};

void* dev_alloc(size_t bytes) {
  if (bytes == 0) bytes = 256;
  ++g_alloc_count;
  int64_t left = g_fail_alloc_after.load();
  while (left >= 0 && !g_fail_alloc_after.compare_exchange_weak(left, left - 1)) {
  }
  if (left == 0)
    throw Error(GBCC_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: injected failure (test hook)");
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(GBCC_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                  cudaGetErrorString(e));
  }
  return p;
}

void dev_free(void* p) {
  if (p) cudaFree(p);
}

namespace {

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

using Extents = std::map<char, int64_t>;

int label_pos(const std::string& lab, char c) {
  auto p = lab.find(c);
  return p == std::string::npos ? -1 : static_cast<int>(p);
}

void check_ix(const Ix& x) {
  if (!x.t) throw Error(GBCC_ERR_STATE, "engine: null tensor");
  if (static_cast<int>(x.lab.size()) != x.t->rank)
    throw Error(GBCC_ERR_STATE, "engine: label count mismatch for " + x.t->name + "(" + x.lab + ")");
}

void add_extents(Extents& e, const Ix& x) {
  check_ix(x);
  for (int k = 0; k < x.t->rank; ++k) {
    char c = x.lab[k];
    auto it = e.find(c);
    if (it == e.end())
      e[c] = x.t->dim[k];
    else if (it->second != x.t->dim[k])
      throw Error(GBCC_ERR_STATE, std::string("engine: extent mismatch for index ") + c + " in " +
                                      x.t->name);
  }
}

int64_t extent_of(const Extents& e, const std::string& labs) {
  int64_t n = 1;
  for (char c : labs) n *= e.at(c);
  return n;
}

int64_t stride_in(const Ix& x, char c) {
  int p = label_pos(x.lab, c);
  return p < 0 ? 0 : x.t->stride(p);
}

// offsets of the composite index over `order` (row-major) into tensor x
std::vector<int64_t> offsets(const std::string& order, const Extents& e, const Ix& x) {
  const int64_t n = extent_of(e, order);
  std::vector<int64_t> out(static_cast<size_t>(n));
  const int d = static_cast<int>(order.size());
  std::vector<int64_t> ext(d), str(d), idx(d, 0);
  for (int k = 0; k < d; ++k) {
    ext[k] = e.at(order[k]);
    str[k] = stride_in(x, order[k]);
  }
  int64_t off = 0;
  for (int64_t i = 0; i < n; ++i) {
    out[static_cast<size_t>(i)] = off;
    for (int k = d - 1; k >= 0; --k) {
      ++idx[k];
      off += str[k];
      if (idx[k] < ext[k]) break;
      off -= str[k] * ext[k];
      idx[k] = 0;
    }
  }
  return out;
}

// labels of `set` in the order they appear in `ref`
std::string order_by(const std::string& set, const std::string& ref) {
  std::string out;
  for (char c : ref)
    if (set.find(c) != std::string::npos) out.push_back(c);
  return out;
}

std::string set_minus(const std::string& a, const std::string& b) {
  std::string out;
  for (char c : a)
    if (b.find(c) == std::string::npos) out.push_back(c);
  return out;
}

std::string set_and(const std::string& a, const std::string& b) {
  std::string out;
  for (char c : a)
    if (b.find(c) != std::string::npos) out.push_back(c);
  return out;
}

// Gather direction: read along R (and transpose in shared memory) when the
// first term is unit-stride along R but not along C.
int pick_transpose(const std::vector<int64_t>& ra, const std::vector<int64_t>& ca) {
  const bool r_unit = ra.size() > 1 && ra[1] - ra[0] == 1;
  const bool c_unit = ca.size() > 1 && ca[1] - ca[0] == 1;
  return (r_unit && !c_unit && ra.size() >= 32) ? 1 : 0;
}

bool same_set(const std::string& a, const std::string& b) {
  std::string x = a, y = b;
  std::sort(x.begin(), x.end());
  std::sort(y.begin(), y.end());
  return x == y;
}

}  // namespace

// ---------------------------------------------------------------------------

struct OperandPlan {
  std::vector<Lin> terms;
  std::string ext;    // ordered external labels (GEMM rows)
  std::string kord;   // ordered contracted labels
  int64_t rows = 0, K = 0;
  bool constant = false;
  bool direct = false;  // FP64: tensor storage used as the panel
  bool inplace = false;  // small-K stream kernel: the one source read in place through its gather tables
  const double* dptr = nullptr;
  int64_t ld = 0;
  GatherArgs gather{};  // packing (FP64 panel or split slices)
  int slices = 0;
  int64_t rows_pad = 0, Kpad = 0;
  __nv_bfloat16* packed = nullptr;  // dedicated split buffer (constants)
  size_t pack_elems = 0;
  // reuse of one split pack by several contractions within a residual
  std::string sig;        // non-empty: sources are not written during a residual
  bool cache_first = false;  // packs into cache_buf
  bool cache_reuse = false;  // reads cache_buf packed by an earlier contraction
  __nv_bfloat16* cache_buf = nullptr;
  // FP64_TC: fixed-point slices under per-row exponents (rows_pad words)
  bool fixed = false;
  unsigned* rowexp = nullptr;
};

// slice pairs of a plan: 3 slices give 6, the fixed-point split's 6 slices 21
constexpr int kMaxPlanPairs = 36;

struct GemmPlan {
  bool use_tc = false;
  bool smallk = false;     // mixed precision, K <= kSmallK: FP32 CUDA-core kernel on FP64 panels
  bool a_is_first = true;  // GEMM M side is the call's A operand
  int64_t M = 0, N = 0, K = 0;
  OperandPlan P[2];        // [0] = M side, [1] = N side
  const int64_t* cm = nullptr;
  const int64_t* cn = nullptr;
  double alpha = 1.0, beta = 0.0;
  double* C = nullptr;
  int slices = 0, npairs = 0, bn = 0;
  bool emu = false;        // FP64_TC: pairs ordered by weight class, one launch per class
  int ksplit = 1;         // K split over CTAs (deterministic two-pass reduction)
  bool m_major = false;   // C unit-stride along M
  int64_t k_per_split = 0;  // FP64: K elements per split; tensor cores: k-blocks per split
  int pa[kMaxPlanPairs] = {}, pb[kMaxPlanPairs] = {};
  double flops = 0.0;
  int sps = 1;             // tensor cores: slices per pipeline stage (2: both slices of a k-block)
  int group = 1;           // tensor cores: M tiles per band of the tile order (1: rows)
  // tensor cores: (tile width, K split, slices per stage, band) candidates
  // for the tuner, the plan's heuristic choice first
  static constexpr int kMaxCand = 24;
  int ncand = 0;
  int cand_bn[kMaxCand] = {}, cand_ks[kMaxCand] = {}, cand_sps[kMaxCand] = {}, cand_group[kMaxCand] = {};
  int64_t cand_kps[kMaxCand] = {};
};

struct Site {
  int kind = 0;  // 0 assign, 1 contract, 2 custom kernels
  TermClass cls = kClassOther;
  GatherArgs gather{};
  GemmPlan plan[3];  // by plan_index(precision)
  cudaEvent_t e0 = nullptr, e1 = nullptr, eg = nullptr;  // profiling: start, end, GEMM start
  bool has_gemm = false;
  std::string label;  // NVTX range name: the operation and its operands
  ~Site() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (eg) cudaEventDestroy(eg);
  }
};

// NVTX ranges around every operation of an EXEC pass when GBCC_NVTX is set in
// the environment (a profiler then shows them; graph replays record none, so
// profile with use_graphs = 0)
static bool nvtx_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GBCC_NVTX");
    return e && *e && std::strcmp(e, "0") != 0;
  }();
  return on;
}

void Engine::prof_begin(Site& s) {
  if (nvtx_enabled()) nvtxRangePushA(s.label.c_str());
  if (!profile_) return;
  if (!s.e0) GBCC_CK(cudaEventCreate(&s.e0));
  if (!s.e1) GBCC_CK(cudaEventCreate(&s.e1));
  if (!s.eg) GBCC_CK(cudaEventCreate(&s.eg));
  GBCC_CK(cudaEventRecord(s.e0, stream_));
  s.has_gemm = false;
}

void Engine::prof_gemm(Site& s) {
  if (!profile_) return;
  GBCC_CK(cudaEventRecord(s.eg, stream_));
  s.has_gemm = true;
}

void Engine::prof_end(Site& s) {
  if (profile_) GBCC_CK(cudaEventRecord(s.e1, stream_));
  if (nvtx_enabled()) nvtxRangePop();
}

std::vector<SiteStat> Engine::site_stats(int precision) {
  std::vector<SiteStat> out;
  GBCC_CK(cudaStreamSynchronize(stream_));
  for (auto& sp : sites_) {
    SiteStat st;
    if (sp->e0 && sp->e1) {
      float ms = 0.f;
      GBCC_CK(cudaEventElapsedTime(&ms, sp->e0, sp->e1));
      st.ms = ms;
      if (sp->has_gemm) {
        GBCC_CK(cudaEventElapsedTime(&ms, sp->eg, sp->e1));
        st.gemm_ms = ms;
      }
    }
    if (sp->kind == 1) {
      const GemmPlan& p = sp->plan[plan_index(precision)];
      st.flops = p.flops;
      st.pairs = p.use_tc ? p.npairs : 0;
      st.classes = p.use_tc && p.emu ? p.slices : 0;
      st.cls = sp->cls;
      st.M = p.M;
      st.N = p.N;
      st.K = p.K;
      st.bn = p.use_tc ? p.bn : (p.smallk ? -1 : 0);
      st.ksplit = p.ksplit;
      st.sps = p.use_tc ? p.sps : 0;
      st.group = p.use_tc ? p.group : 0;
    } else {
      st.M = sp->gather.R;
      st.N = sp->gather.C;
    }
    out.push_back(st);
  }
  return out;
}

Engine::Engine() = default;

Engine::~Engine() {
  for (void* p : owned_) dev_free(p);
  for (auto& kv : tensors_) dev_free(kv.second->d);
  dev_free(w64a_);
  dev_free(w64b_);
  dev_free(wbfa_);
  dev_free(wbfb_);
  dev_free(wpart_);
}

Tensor& Engine::tensor(const std::string& name, std::initializer_list<int64_t> dims, bool constant) {
  auto it = tensors_.find(name);
  if (it != tensors_.end()) {
    Tensor& t = *it->second;
    int k = 0;
    bool same = static_cast<int>(dims.size()) == t.rank;
    for (int64_t dval : dims) same = same && (k < t.rank && t.dim[k++] == dval);
    if (!same) throw Error(GBCC_ERR_STATE, "engine: tensor " + name + " re-requested with new shape");
    return t;
  }
  auto t = std::make_unique<Tensor>();
  t->name = name;
  t->rank = static_cast<int>(dims.size());
  int k = 0;
  for (int64_t dval : dims) t->dim[k++] = dval;
  t->constant = constant;
  const size_t bytes = static_cast<size_t>(t->size()) * sizeof(double);
  t->d = static_cast<double*>(dev_alloc(bytes));
  GBCC_CK(cudaMemsetAsync(t->d, 0, bytes, stream_));
  bytes_ += bytes;
  Tensor& ref = *t;
  tensors_[name] = std::move(t);
  return ref;
}

void Engine::release(Tensor& t) {
  if (!t.d) return;
  GBCC_CK(cudaStreamSynchronize(stream_));
  dev_free(t.d);
  t.d = nullptr;
  bytes_ -= static_cast<size_t>(t.size()) * sizeof(double);
}

void Engine::acquire(Tensor& t) {
  if (t.d) return;
  const size_t bytes = static_cast<size_t>(t.size()) * sizeof(double);
  t.d = static_cast<double*>(dev_alloc(bytes));
  GBCC_CK(cudaMemsetAsync(t.d, 0, bytes, stream_));
  bytes_ += bytes;
}

Tensor* Engine::find(const std::string& name) {
  auto it = tensors_.find(name);
  return it == tensors_.end() ? nullptr : it->second.get();
}

void Engine::reset_plans() {
  pack_uses_.clear();
  sites_.clear();
  for (void* p : owned_) dev_free(p);
  owned_.clear();
  planned_ = false;
  ws64_a_ = ws64_b_ = wsbf_a_ = wsbf_b_ = wspart_ = 0;
  dev_free(wpart_);
  wpart_ = nullptr;
  dev_free(w64a_);
  dev_free(w64b_);
  dev_free(wbfa_);
  dev_free(wbfb_);
  w64a_ = w64b_ = nullptr;
  wbfa_ = wbfb_ = nullptr;
}

void Engine::begin(Mode m, int precision) {
  if (m == Mode::kExec && !planned_) throw Error(GBCC_ERR_STATE, "engine: EXEC before PLAN");
  mode_ = m;
  prec_ = precision;
  cursor_ = 0;
  flops_ = 0.0;
  n_tc_ = 0;
  n_launch_ = 0;
}

void Engine::end() {
  if (mode_ == Mode::kPlan) {
    planned_ = true;
  } else if (cursor_ != sites_.size()) {
    throw Error(GBCC_ERR_STATE, "engine: program ended early");
  }
}

Site& Engine::site() {
  if (mode_ == Mode::kPlan) {
    sites_.push_back(std::make_unique<Site>());
    ++cursor_;
    return *sites_.back();
  }
  if (cursor_ >= sites_.size()) throw Error(GBCC_ERR_STATE, "engine: program longer than its plan");
  return *sites_[cursor_++];
}

DevTable Engine::upload(const std::vector<int64_t>& v) {
  DevTable t;
  t.n = static_cast<int64_t>(v.size());
  const size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(int64_t);
  t.d = static_cast<int64_t*>(dev_alloc(bytes));
  owned_.push_back(t.d);
  bytes_ += bytes;
  if (!v.empty()) GBCC_CK(cudaMemcpy(t.d, v.data(), v.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  return t;
}

int Engine::slices_for(TermClass cls, double flops) const {
  // contractions this small are cheaper in FP64 than a tensor-core launch
  if (flops < 1.0e6) return 0;
  return slices_[cls];
}

// ---------------------------------------------------------------------------

void Engine::assign(const Ix& c, double beta, const std::vector<Factor>& terms) {
  Site& s = site();
  if (mode_ == Mode::kExec) {
    if (s.kind != 0) throw Error(GBCC_ERR_STATE, "engine: site kind mismatch");
    prof_begin(s);
    launch_gather(s.gather, stream_);
    ++n_launch_;
    prof_end(s);
    return;
  }
  s.kind = 0;
  s.label = "assign " + c.t->name + "(" + c.lab + ")";
  check_ix(c);
  if (terms.empty() || terms.size() > static_cast<size_t>(kMaxTerms))
    throw Error(GBCC_ERR_STATE, "engine: assign needs 1..4 terms");
  Extents e;
  add_extents(e, c);
  for (const auto& f : terms) {
    add_extents(e, f.a);
    if (f.b.t) add_extents(e, f.b);
    for (char ch : f.a.lab)
      if (c.lab.find(ch) == std::string::npos)
        throw Error(GBCC_ERR_STATE, std::string("engine: assign index ") + ch + " not in output");
    for (char ch : f.b.lab)
      if (c.lab.find(ch) == std::string::npos)
        throw Error(GBCC_ERR_STATE, std::string("engine: assign index ") + ch + " not in output");
  }
  // split output dims into rows [0,split) and columns [split,rank)
  const int rank = c.t->rank;
  int split = rank;
  int64_t cols = 1;
  while (split > 0 && cols < 1024) {
    --split;
    cols *= c.t->dim[split];
  }
  const std::string rlab = c.lab.substr(0, split), clab = c.lab.substr(split);
  GatherArgs& g = s.gather;
  std::memset(&g, 0, sizeof(g));
  g.nterms = static_cast<int>(terms.size());
  for (size_t t = 0; t < terms.size(); ++t) {
    GatherTerm& T = g.t[t];
    gather_set_coef(T, terms[t].coef);
    T.a = terms[t].a.t->d;
    const std::vector<int64_t> hra = offsets(rlab, e, terms[t].a), hca = offsets(clab, e, terms[t].a);
    if (t == 0) g.transpose = pick_transpose(hra, hca);
    gather_set_c4(T, hca.data(), static_cast<int64_t>(hca.size()));
    T.ra = upload(hra).d;
    T.ca = upload(hca).d;
    if (terms[t].b.t) {
      g.products = 1;
      T.b = terms[t].b.t->d;
      T.rb = upload(offsets(rlab, e, terms[t].b)).d;
      T.cb = upload(offsets(clab, e, terms[t].b)).d;
    }
  }
  g.R = g.Rpad = extent_of(e, rlab);
  g.C = g.Cpad = extent_of(e, clab);
  g.out = c.t->d;
  g.ldo = g.C;
  g.beta = beta;
  gather_finish(g);
}

// ---------------------------------------------------------------------------

namespace {

bool storage_is_panel(const Ix& x, const std::string& ext) {
  // storage order = [ext labels...][K labels...]
  const int ne = static_cast<int>(ext.size());
  for (int k = 0; k < x.t->rank; ++k) {
    const bool is_ext = ext.find(x.lab[k]) != std::string::npos;
    if ((k < ne) != is_ext) return false;
  }
  return true;
}

}  // namespace

// The split panel of one operand of a tensor-core contraction: its constant
// pack, the pack cache, or a fresh pack into the workspace.
__nv_bfloat16* Engine::tc_panel(OperandPlan& op, int side) {
  if (op.constant) {
    if (!op.packed) throw Error(GBCC_ERR_STATE, "engine: constant operand not packed");
    return op.packed;
  }
  if (op.cache_reuse) return op.cache_buf;
  __nv_bfloat16* out = op.cache_first ? op.cache_buf : (side == 0 ? wbfa_ : wbfb_);
  pack_panel(op, out);
  return out;
}

// Split pack of an operand into `out`: one gather, or for fixed-point slices
// the row exponents (zeroed, then the exponent pass) and the digit pass.
void Engine::pack_panel(const OperandPlan& op, __nv_bfloat16* out) {
  GatherArgs g = op.gather;
  g.outs = out;
  if (op.fixed) {
    GBCC_CK(cudaMemsetAsync(op.rowexp, 0, static_cast<size_t>(op.rows_pad) * sizeof(unsigned), stream_));
    g.fixed = 1;
    launch_gather(g, stream_);
    g.fixed = 2;
    ++n_launch_;  // the exponent pass (the memset is not a kernel)
  }
  launch_gather(g, stream_);
  ++n_launch_;
}

GemmTcArgs Engine::tc_args(const GemmPlan& p, TermClass cls, __nv_bfloat16* const panel[2]) const {
  GemmTcArgs t{};
  t.M = p.M;
  t.N = p.N;
  t.Mpad = p.P[0].rows_pad;
  t.Npad = round_up(p.N, p.bn);
  t.a_rows = p.P[0].rows_pad;
  t.b_rows = p.P[1].rows_pad;  // padded for every candidate tile width
  t.Kpad = p.P[0].Kpad;
  t.A = panel[0];
  t.a_slices = p.slices;
  t.B = panel[1];
  t.b_slices = p.slices;
  // a slice limit below the packed count keeps the pairs p + q < limit: the
  // split is sequential, so these are exactly the products of a
  // limit-slice split (used to measure the error of fewer slices); it
  // applies to the mixed plan only
  const int lim = p.emu ? 0 : slice_limit_[cls];
  t.npairs = 0;
  // FP64_TC: the pairs of each weight class are set per launch (launch_tc_classes)
  for (int q = 0; q < (p.emu ? 0 : p.npairs); ++q) {
    if (lim > 0 && p.pa[q] + p.pb[q] >= lim) continue;
    t.pa[t.npairs] = p.pa[q];
    t.pb[t.npairs] = p.pb[q];
    ++t.npairs;
  }
  t.C = p.C;
  t.cm = p.cm;
  t.cn = p.cn;
  t.alpha = p.alpha;
  t.beta = p.beta;
  t.bn = p.bn;
  // the accumulation length of the slice count in effect (a calibration trial
  // under a slice limit measures the error the smaller plan will have)
  const int eff_slices = (lim > 0 && lim < p.slices) ? lim : p.slices;
  t.chunk = eff_slices >= 3 ? chunk_ : chunk_lo_;
  if (p.emu) {
    // exact FP32 chunk sums: 4 steps of 64 products below 2^14 units each,
    // two chunks per FP32 register sum before the float-float fold
    t.chunk = kFixedChunk;
    t.fold = kFixedFold;
  }
  t.err = err_;
  t.ksplit = p.ksplit;
  t.kb_per_split = static_cast<int>(p.k_per_split);
  t.partial = wpart_;
  t.m_major = p.m_major ? 1 : 0;
  // a slice limit makes the packed slices a superset of the used ones: one
  // pair per stage then
  t.sps = (lim > 0 && lim < p.slices) ? 1 : p.sps;
  t.group = p.group;
  return t;
}

void Engine::launch_tc(const GemmPlan& p, const GemmTcArgs& t) {
  if (!launch_gemm_tc(t, stream_)) throw Error(GBCC_ERR_CUDA, "tcgen05 GEMM launch rejected (tensor map or size)");
  ++n_tc_;
  ++tc_total_;
  ++n_launch_;
  if (p.ksplit > 1) {
    launch_splitk_reduce(p.M, p.N, p.ksplit, wpart_, t.Mpad, t.Npad, p.C, p.cm, p.cn, t.alpha, t.beta, stream_);
    ++n_launch_;
  }
}

// FP64_TC: one launch per weight class w = p + q, the classes of the smallest
// weight first; the first applies the call's beta, the rest accumulate.
void Engine::launch_tc_classes(const GemmPlan& p, TermClass cls, __nv_bfloat16* const panel[2]) {
  GemmTcArgs t = tc_args(p, cls, panel);
  for (int w = p.slices - 1; w >= 0; --w) {
    t.npairs = fixed_class_pairs(p.slices, w, t.pa, t.pb);
    t.beta = w == p.slices - 1 ? p.beta : 1.0;
    launch_tc(p, t);
  }
}

// Tile width and K split of every tensor-core contraction chosen by timing
// its candidates (plan-time lists) on its own operands: each candidate runs
// once untimed and `reps` times between CUDA events, the fastest is kept.
// The outputs of the timed launches are scratch (a residual recomputes them).
void Engine::autotune(int reps) {
  if (!planned_) throw Error(GBCC_ERR_STATE, "engine: autotune before PLAN");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  GBCC_CK(cudaEventCreate(&e0));
  GBCC_CK(cudaEventCreate(&e1));
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } ev{e0, e1};
  for (auto& sp : sites_) {
    if (sp->kind != 1) continue;
    GemmPlan& p = sp->plan[1];
    if (!p.use_tc || p.ncand < 2) continue;
    // shape key: SM count, class, M x N x K, slices, output orientation
    const std::string key = std::to_string(num_sms()) + ":c" + std::to_string(static_cast<int>(sp->cls)) + ":" +
                            std::to_string(p.M) + "x" + std::to_string(p.N) + "x" + std::to_string(p.K) + ":s" +
                            std::to_string(p.slices) + (p.m_major ? ":m" : ":n");
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = tune_table().find(key);
      int hit = -1;
      if (it != tune_table().end())
        for (int c = 0; c < p.ncand && hit < 0; ++c)
          if (p.cand_bn[c] == it->second.bn && p.cand_ks[c] == it->second.ksplit &&
              p.cand_kps[c] == it->second.kps && p.cand_sps[c] == it->second.sps &&
              p.cand_group[c] == it->second.group)
            hit = c;
      if (hit >= 0) {
        p.bn = p.cand_bn[hit];
        p.ksplit = p.cand_ks[hit];
        p.k_per_split = p.cand_kps[hit];
        p.sps = p.cand_sps[hit];
        p.group = p.cand_group[hit];
        continue;
      }
    }
    __nv_bfloat16* panel[2];
    for (int side = 0; side < 2; ++side) panel[side] = tc_panel(p.P[side], side);
    float best = 0.f;
    int pick = -1;
    for (int c = 0; c < p.ncand; ++c) {
      GemmPlan q = p;
      q.bn = p.cand_bn[c];
      q.ksplit = p.cand_ks[c];
      q.k_per_split = p.cand_kps[c];
      q.sps = p.cand_sps[c];
      q.group = p.cand_group[c];
      const GemmTcArgs t = tc_args(q, sp->cls, panel);
      if (!launch_gemm_tc(t, stream_)) continue;
      ++tc_total_;
      if (q.ksplit > 1)
        launch_splitk_reduce(q.M, q.N, q.ksplit, wpart_, t.Mpad, t.Npad, q.C, q.cm, q.cn, q.alpha, q.beta, stream_);
      GBCC_CK(cudaEventRecord(e0, stream_));
      for (int r = 0; r < reps; ++r) launch_tc(q, t);
      GBCC_CK(cudaEventRecord(e1, stream_));
      GBCC_CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      GBCC_CK(cudaEventElapsedTime(&ms, e0, e1));
      if (pick < 0 || ms < best) {
        best = ms;
        pick = c;
      }
    }
    if (pick >= 0) {
      p.bn = p.cand_bn[pick];
      p.ksplit = p.cand_ks[pick];
      p.k_per_split = p.cand_kps[pick];
      p.sps = p.cand_sps[pick];
      p.group = p.cand_group[pick];
      std::lock_guard<std::mutex> lk(g_tune_mu);
      tune_table()[key] = TuneChoice{p.bn, p.ksplit, p.sps, p.group, p.k_per_split};
    }
  }
  GBCC_CK(cudaStreamSynchronize(stream_));
}

void Engine::custom(const std::function<void(cudaStream_t)>& fn, int launches) {
  Site& s = site();
  if (mode_ == Mode::kExec) {
    if (s.kind != 2) throw Error(GBCC_ERR_STATE, "engine: site kind mismatch");
    prof_begin(s);
    fn(stream_);
    n_launch_ += launches;
    prof_end(s);
    return;
  }
  s.kind = 2;
  s.label = "kernels (site " + std::to_string(sites_.size() - 1) + ")";
}

void Engine::contract(const Ix& c, double beta, double alpha, const std::vector<Lin>& A,
                      const std::vector<Lin>& B, TermClass cls) {
  Site& s = site();
  if (mode_ == Mode::kExec) {
    if (s.kind != 1) throw Error(GBCC_ERR_STATE, "engine: site kind mismatch");
    GemmPlan& p = s.plan[plan_index(prec_)];
    flops_ += p.flops;
    prof_begin(s);
    if (p.use_tc) {
      __nv_bfloat16* panel[2];
      for (int side = 0; side < 2; ++side) panel[side] = tc_panel(p.P[side], side);
      prof_gemm(s);
      if (p.emu) {
        launch_tc_classes(p, cls, panel);
      } else {
        const GemmTcArgs t = tc_args(p, cls, panel);
        launch_tc(p, t);
      }
    } else {
      const double* panel[2];
      for (int side = 0; side < 2; ++side) {
        OperandPlan& op = p.P[side];
        if (op.direct) {
          panel[side] = op.dptr;
        } else if (op.inplace) {
          panel[side] = op.gather.t[0].a;
        } else {
          double* w = side == 0 ? w64a_ : w64b_;
          GatherArgs g = op.gather;
          g.out = w;
          launch_gather(g, stream_);
          ++n_launch_;
          panel[side] = w;
        }
      }
      GemmF64Args f{};
      f.M = p.M;
      f.N = p.N;
      f.K = p.K;
      f.A = panel[0];
      f.lda = p.P[0].direct ? p.P[0].ld : p.K;
      f.B = panel[1];
      f.ldb = p.P[1].direct ? p.P[1].ld : p.K;
      f.C = p.C;
      f.cm = p.cm;
      f.cn = p.cn;
      f.alpha = p.alpha;
      f.beta = p.beta;
      f.ksplit = p.ksplit;
      f.k_per_split = p.k_per_split;
      f.partial = wpart_;
      f.m_major = p.m_major ? 1 : 0;
      if (p.P[0].inplace) {
        f.a_ra = p.P[0].gather.t[0].ra;
        f.a_ca = p.P[0].gather.t[0].ca;
        f.lda = 0;
      }
      prof_gemm(s);
      if (p.smallk) {
        if (!launch_gemm_smallk(f, stream_)) throw Error(GBCC_ERR_STATE, "engine: in-place small-K operand off the stream kernel");
        ++n_launch_;
      } else {
        launch_gemm_f64(f, stream_);
        n_launch_ += p.ksplit > 1 ? 2 : 1;
      }
    }
    prof_end(s);
    return;
  }

  // ---------------- PLAN ----------------
  s.kind = 1;
  s.cls = cls;
  check_ix(c);
  static const char* const kClassName[3] = {"ladder", "ring", "other"};
  s.label = "contract " + c.t->name + "(" + c.lab + ") <- " + A.at(0).x.t->name + "(" + A.at(0).x.lab + ") " +
            B.at(0).x.t->name + "(" + B.at(0).x.lab + ") [" + kClassName[static_cast<int>(cls)] + "]";
  if (A.empty() || B.empty() || A.size() > static_cast<size_t>(kMaxTerms) ||
      B.size() > static_cast<size_t>(kMaxTerms))
    throw Error(GBCC_ERR_STATE, "engine: contract needs 1..4 terms per operand");
  Extents e;
  add_extents(e, c);
  for (const auto* ops : {&A, &B})
    for (const auto& l : *ops) {
      add_extents(e, l.x);
      if (l.y.t) add_extents(e, l.y);
    }
  // the first term of an operand is a single factor carrying all its indices
  auto term_labels = [](const Lin& l) { return l.y.t ? l.x.lab + l.y.lab : l.x.lab; };
  if (A[0].y.t || B[0].y.t) throw Error(GBCC_ERR_STATE, "engine: the first operand term must be one factor");
  for (const auto& l : A)
    if (!same_set(term_labels(l), A[0].x.lab)) throw Error(GBCC_ERR_STATE, "engine: A terms differ in indices");
  for (const auto& l : B)
    if (!same_set(term_labels(l), B[0].x.lab)) throw Error(GBCC_ERR_STATE, "engine: B terms differ in indices");
  const std::string la = A[0].x.lab, lb = B[0].x.lab;
  const std::string kset = set_and(la, lb);
  const std::string aext = set_minus(la, kset), bext = set_minus(lb, kset);
  for (char ch : kset)
    if (c.lab.find(ch) != std::string::npos)
      throw Error(GBCC_ERR_STATE, "engine: Hadamard indices are not supported");
  if (!same_set(aext + bext, c.lab))
    throw Error(GBCC_ERR_STATE, "engine: output indices must be exactly the external ones (" + c.lab + ")");
  const int64_t rowsA = extent_of(e, aext), rowsB = extent_of(e, bext), K = extent_of(e, kset);
  bool constA = true, constB = true;
  for (const auto& l : A) constA = constA && l.x.t->constant && (!l.y.t || l.y.t->constant);
  for (const auto& l : B) constB = constB && l.x.t->constant && (!l.y.t || l.y.t->constant);
  const double flops = 2.0 * static_cast<double>(rowsA) * rowsB * K;

  for (int pm = 0; pm < (emu_ ? 3 : 2); ++pm) {
    GemmPlan& p = s.plan[pm];
    p = GemmPlan{};
    p.flops = flops;
    const bool emu = pm == 2;
    int slices = pm == 1 ? slices_for(cls, flops) : (emu && slices_for(cls, flops) > 0 ? kFixedSlices : 0);
    // a short contraction into a large output is memory-bound: CUDA cores
    // (measured faster for N > 32; the tensor-core kernel wins below).  The
    // FP64-grade plan keeps such contractions on the FP64 kernel.
    if (slices > 0 && !emu && K <= kSmallK && std::min(rowsA, rowsB) >= 32 &&
        static_cast<double>(rowsA) * static_cast<double>(rowsB) >= 1048576.0) {
      slices = 0;
      p.smallk = true;
    }
    // the larger operand on M: it is then re-read once per N tile, and N
    // tiles are up to 256 wide (less padding alone, with the large operand on
    // N, measured slower: more L2 re-reads of it)
    p.a_is_first = rowsA >= rowsB;
    const std::vector<Lin>& Ms = p.a_is_first ? A : B;
    const std::vector<Lin>& Ns = p.a_is_first ? B : A;
    const std::string mext = p.a_is_first ? aext : bext;
    const std::string next = p.a_is_first ? bext : aext;
    const bool constM = p.a_is_first ? constA : constB;
    const bool constN = p.a_is_first ? constB : constA;
    p.M = extent_of(e, mext);
    p.N = extent_of(e, next);
    p.K = K;
    p.beta = beta;
    p.C = c.t->d;
    p.use_tc = slices > 0;
    OperandPlan& PM = p.P[0];
    OperandPlan& PN = p.P[1];
    PM.terms = Ms;
    PN.terms = Ns;
    PM.constant = constM;
    PN.constant = constN;
    PM.rows = p.M;
    PN.rows = p.N;
    PM.K = PN.K = K;
    PM.ext = order_by(mext, c.lab);
    PN.ext = order_by(next, c.lab);
    // contracted-index order
    const Ix& bigM = Ms[0].x;
    const Ix& bigN = Ns[0].x;
    if (!p.use_tc) {
      const bool dM = Ms.size() == 1 && !Ms[0].y.t && storage_is_panel(bigM, mext);
      const bool dN = Ns.size() == 1 && !Ns[0].y.t && storage_is_panel(bigN, next);
      if (dM && (!dN || bigM.t->size() >= bigN.t->size())) {
        PM.direct = true;
        PM.ext = order_by(mext, bigM.lab);
        PM.kord = order_by(kset, bigM.lab);
        if (dN && order_by(kset, bigN.lab) == PM.kord) {
          PN.direct = true;
          PN.ext = order_by(next, bigN.lab);
        }
      } else if (dN) {
        PN.direct = true;
        PN.ext = order_by(next, bigN.lab);
        PM.kord = order_by(kset, bigN.lab);
      } else {
        const Ix& ref = bigM.t->size() >= bigN.t->size() ? bigM : bigN;
        PM.kord = order_by(kset, ref.lab);
      }
    } else {
      // pack reads are cheapest along the storage order of the per-iteration operand
      const Ix* ref = nullptr;
      if (!constM && !constN) ref = bigM.t->size() >= bigN.t->size() ? &bigM : &bigN;
      else if (!constM) ref = &bigM;
      else if (!constN) ref = &bigN;
      else ref = &bigM;
      PM.kord = order_by(kset, ref->lab);
    }
    PN.kord = PM.kord;
    double coef_direct = 1.0;
    for (int side = 0; side < 2; ++side) {
      OperandPlan& op = p.P[side];
      if (op.direct) {
        op.dptr = op.terms[0].x.t->d;
        op.ld = op.K;
        coef_direct *= op.terms[0].coef;
        continue;
      }
      GatherArgs& g = op.gather;
      std::memset(&g, 0, sizeof(g));
      g.nterms = static_cast<int>(op.terms.size());
      // a single one-factor term packs as a plain copy; its coefficient scales alpha
      const bool single = op.terms.size() == 1 && !op.terms[0].y.t;
      if (single) coef_direct *= op.terms[0].coef;
      g.plain = single ? 1 : 0;
      for (size_t t = 0; t < op.terms.size(); ++t) {
        gather_set_coef(g.t[t], single ? 1.0 : op.terms[t].coef);
        g.t[t].a = op.terms[t].x.t->d;
        const std::vector<int64_t> hra = offsets(op.ext, e, op.terms[t].x), hca = offsets(op.kord, e, op.terms[t].x);
        if (t == 0) g.transpose = pick_transpose(hra, hca);
        gather_set_c4(g.t[t], hca.data(), static_cast<int64_t>(hca.size()));
        g.t[t].ra = upload(hra).d;
        g.t[t].ca = upload(hca).d;
        if (op.terms[t].y.t) {
          g.products = 1;
          g.t[t].b = op.terms[t].y.t->d;
          g.t[t].rb = upload(offsets(op.ext, e, op.terms[t].y)).d;
          g.t[t].cb = upload(offsets(op.kord, e, op.terms[t].y)).d;
        }
      }
      gather_finish(g);
      g.R = op.rows;
      g.C = op.K;
      if (!p.use_tc) {
        g.Rpad = op.rows;
        g.Cpad = op.K;
        g.ldo = op.K;
        g.beta = 0.0;
        size_t need = static_cast<size_t>(op.rows * op.K);
        if (side == 0) ws64_a_ = std::max(ws64_a_, need);
        else ws64_b_ = std::max(ws64_b_, need);
      }
    }
    p.alpha = alpha * coef_direct;
    {
      Ix cx = c;
      const std::vector<int64_t> hm = offsets(p.P[0].ext, e, cx), hn = offsets(p.P[1].ext, e, cx);
      // epilogue lane direction: along M when C is unit-stride in M but not in N
      const bool m_unit = hm.size() > 1 && hm[1] - hm[0] == 1;
      const bool n_unit = hn.size() > 1 && hn[1] - hn[0] == 1;
      p.m_major = m_unit && !n_unit;
      p.cm = upload(hm).d;
      p.cn = upload(hn).d;
    }
    // a single-factor M operand contiguous along M (its pack would transpose)
    // is read in place by the stream kernel: no FP64 panel written and read back
    if (p.smallk && !p.P[0].direct && p.P[0].gather.plain && p.P[0].gather.transpose &&
        smallk_streams(p.N, K, p.m_major))
      p.P[0].inplace = true;
    if (!p.use_tc && !p.smallk) {
      // fewer 64 x 64 output tiles than two per SM: split K over blocks (one SM
      // runs FP64 at ~1/150 of the GPU's already low FP64 rate, so even a
      // 1 MFLOP contraction is slow on a single block)
      const int64_t tiles = ((p.M + 63) / 64) * ((p.N + 63) / 64);
      const int64_t sms = num_sms();
      if (tiles < 2 * sms && K >= 32) {
        int64_t ks = std::min<int64_t>((2 * sms + tiles - 1) / tiles, K / 16);
        if (ks > 1) {
          int64_t kps = (K + ks - 1) / ks;
          kps = (kps + 15) / 16 * 16;
          ks = (K + kps - 1) / kps;
          p.ksplit = static_cast<int>(ks);
          p.k_per_split = kps;
          wspart_ = std::max(wspart_, static_cast<size_t>(ks * p.M * p.N));
        }
      }
    }
    if (p.use_tc) {
      p.slices = slices;
      p.emu = emu;
      // the ladder and ring contractions take the faster 192/256-wide tiles
      // (not FP64_TC: its chunk sums need the float-float fold of tiles up to 128)
      const bool wide = !emu && (cls == kClassLadder || cls == kClassRing);
      p.bn = gemm_tc_pick_bn(p.N, wide);
      int bns[4];
      const int nbn = gemm_tc_bn_candidates(p.N, wide, bns);
      int64_t npanel = 0;  // N-side panel rows: room for every candidate tile width
      for (int c = 0; c < nbn; ++c) npanel = std::max<int64_t>(npanel, round_up(p.N, bns[c]));
      p.npairs = 0;
      if (emu) {
        for (int w = 0; w < slices; ++w) p.npairs += fixed_class_pairs(slices, w, p.pa + p.npairs, p.pb + p.npairs);
      } else {
        for (int a = 0; a < slices; ++a)
          for (int b = 0; b < slices; ++b)
            if (a + b < slices) {
              p.pa[p.npairs] = a;
              p.pb[p.npairs] = b;
              ++p.npairs;
            }
      }
      const int64_t Kpad = round_up(std::max<int64_t>(K, 1), kTcBK);
      for (int side = 0; side < 2; ++side) {
        OperandPlan& op = p.P[side];
        op.slices = slices;
        op.Kpad = Kpad;
        op.rows_pad = side == 0 ? round_up(op.rows, kTcBM) : npanel;
        GatherArgs& g = op.gather;
        g.Rpad = op.rows_pad;
        g.Cpad = Kpad;
        g.ldo = Kpad;
        g.out = nullptr;
        g.nslices = slices;
        g.slice_stride = op.rows_pad * Kpad;
        if (emu) {
          op.fixed = true;
          op.rowexp = static_cast<unsigned*>(dev_alloc(static_cast<size_t>(op.rows_pad) * sizeof(unsigned)));
          owned_.push_back(op.rowexp);
          bytes_ += static_cast<size_t>(op.rows_pad) * sizeof(unsigned);
          g.rowexp = op.rowexp;
          g.fixed = 2;
        }
        const size_t need = static_cast<size_t>(slices) * op.rows_pad * Kpad;
        if (!op.constant) {
          bool frozen = true;
          std::string sig;
          for (const auto& l : op.terms) {
            frozen = frozen && frozen_.count(l.x.t) > 0 && (!l.y.t || frozen_.count(l.y.t) > 0);
            // a single one-factor term is packed unscaled (plain copy)
            const double coef = (op.terms.size() == 1 && !l.y.t) ? 1.0 : l.coef;
            sig += l.x.t->name + "(" + l.x.lab + ")";
            if (l.y.t) sig += l.y.t->name + "(" + l.y.lab + ")";
            sig += "*" + std::to_string(coef) + ";";
          }
          if (frozen) {
            op.sig = sig + op.ext + "|" + op.kord + "|" + (emu ? "fixed" : "float") + std::to_string(slices) + "|" +
                     std::to_string(op.rows_pad) + "|" + std::to_string(Kpad);
            op.pack_elems = need;
            pack_uses_[op.sig].push_back(&op);
          }
        }
        if (op.constant) {
          op.pack_elems = need;  // allocated and packed by prepack()
        } else if (side == 0) {
          wsbf_a_ = std::max(wsbf_a_, need);
        } else {
          wsbf_b_ = std::max(wsbf_b_, need);
        }
      }
      // fewer output tiles than SMs and a long K: split K over CTAs.  The
      // candidates: every tile width with that split, and unsplit where it splits
      const int64_t kblocks = Kpad / kTcBK;
      const int64_t sms = num_sms();
      p.ncand = 0;
      for (int c = 0; c < nbn; ++c) {
        const int64_t npad = round_up(p.N, bns[c]);
        const int64_t tiles = (p.P[0].rows_pad / kTcBM) * (npad / bns[c]);
        int64_t ks = 1, kbps = 0;
        if (tiles < sms && kblocks >= 16) {
          ks = std::min<int64_t>((sms + tiles - 1) / tiles, kblocks / 8);
        } else if (tiles < 3 * sms && kblocks >= 64) {
          // one to three waves: a split that fills the last wave better (the
          // Giabc pair products at o = 32, v = 320: 240 tiles on 152 SMs fill
          // 79 % of two waves, split in three 95 % of five)
          auto fill = [&](int64_t k) {
            const int64_t n = tiles * k;
            return static_cast<double>(n) / static_cast<double>((n + sms - 1) / sms * sms);
          };
          double best = fill(1) + 0.05;
          for (int64_t k = 2; k <= 4 && kblocks / k >= 16; ++k)
            if (fill(k) > best) {
              best = fill(k);
              ks = k;
            }
        }
        if (ks > 1) {
          kbps = (kblocks + ks - 1) / ks;
          ks = (kblocks + kbps - 1) / kbps;
        } else {
          ks = 1;
        }
        if (ks > 1) wspart_ = std::max(wspart_, static_cast<size_t>(ks * p.P[0].rows_pad * npad));
        // both slices of a k-block per stage: two slices, tiles up to 192 wide
        const int nsps = (slices == 2 && bns[c] >= 64 && bns[c] <= 192) ? 2 : 1;
        // bands of 8 M tiles: many N tiles per row and enough rows
        const bool banded = npad / bns[c] >= 8 && p.P[0].rows_pad / kTcBM >= 16;
        for (int sp = 1; sp <= nsps; ++sp) {
          for (int split = 0; split < (ks > 1 ? 2 : 1); ++split) {
            for (int band = 0; band < (banded && (split == 1 || ks == 1) ? 2 : 1); ++band) {
              if (p.ncand >= GemmPlan::kMaxCand) break;
              p.cand_bn[p.ncand] = bns[c];
              p.cand_ks[p.ncand] = split == 0 ? static_cast<int>(ks) : 1;
              p.cand_kps[p.ncand] = split == 0 ? kbps : 0;
              p.cand_sps[p.ncand] = sp;
              p.cand_group[p.ncand] = band ? 8 : 1;
              ++p.ncand;
            }
          }
        }
      }
      // the heuristic choice: the first candidate
      p.bn = p.cand_bn[0];
      p.ksplit = p.cand_ks[0];
      p.k_per_split = p.cand_kps[0];
      p.sps = p.cand_sps[0];
      p.group = p.cand_group[0];
    }
  }
}

void Engine::finalize() {
  if (!planned_) throw Error(GBCC_ERR_STATE, "engine: finalize before PLAN");
  // every old workspace is released and its pointer cleared before the first
  // new allocation: one that fails leaves no pointer to freed memory behind
  for (void** p : {reinterpret_cast<void**>(&w64a_), reinterpret_cast<void**>(&w64b_),
                   reinterpret_cast<void**>(&wbfa_), reinterpret_cast<void**>(&wbfb_),
                   reinterpret_cast<void**>(&wpart_)}) {
    dev_free(*p);
    *p = nullptr;
  }
  w64a_ = static_cast<double*>(dev_alloc(ws64_a_ * sizeof(double)));
  w64b_ = static_cast<double*>(dev_alloc(ws64_b_ * sizeof(double)));
  wbfa_ = static_cast<__nv_bfloat16*>(dev_alloc(wsbf_a_ * sizeof(__nv_bfloat16)));
  wbfb_ = static_cast<__nv_bfloat16*>(dev_alloc(wsbf_b_ * sizeof(__nv_bfloat16)));
  wpart_ = static_cast<double*>(dev_alloc(wspart_ * sizeof(double)));
  bytes_ += (ws64_a_ + ws64_b_ + wspart_) * sizeof(double) + (wsbf_a_ + wsbf_b_) * sizeof(__nv_bfloat16);
  // packs shared by several contractions of a residual get their own buffer
  for (auto& kv : pack_uses_) {
    if (kv.second.size() < 2) continue;
    OperandPlan* first = kv.second.front();
    if (!first->cache_buf) {
      first->cache_buf = static_cast<__nv_bfloat16*>(dev_alloc(first->pack_elems * sizeof(__nv_bfloat16)));
      owned_.push_back(first->cache_buf);
      bytes_ += first->pack_elems * sizeof(__nv_bfloat16);
    }
    first->cache_first = true;
    for (size_t i = 1; i < kv.second.size(); ++i) {
      kv.second[i]->cache_reuse = true;
      kv.second[i]->cache_buf = first->cache_buf;
    }
  }
  packed_[0] = packed_[1] = packed_[2] = false;
}

void Engine::prepack(int precision) {
  const int pi = plan_index(precision);
  if (!planned_) throw Error(GBCC_ERR_STATE, "engine: prepack before PLAN");
  if (pi == 0 || packed_[pi]) return;
  if (pi == 2 && !emu_) throw Error(GBCC_ERR_STATE, "engine: no FP64_TC plan");
  for (auto& sp : sites_) {
    if (sp->kind != 1) continue;
    GemmPlan& p = sp->plan[pi];
    if (!p.use_tc) continue;
    for (int side = 0; side < 2; ++side) {
      OperandPlan& op = p.P[side];
      if (!op.constant) continue;
      if (!op.packed) {
        op.packed = static_cast<__nv_bfloat16*>(dev_alloc(op.pack_elems * sizeof(__nv_bfloat16)));
        owned_.push_back(op.packed);
        bytes_ += op.pack_elems * sizeof(__nv_bfloat16);
      }
      pack_panel(op, op.packed);
    }
  }
  GBCC_CK(cudaGetLastError());
  packed_[pi] = true;
}

}  // namespace gbcc

extern "C" int gbcc_testing_fail_alloc(int64_t after, int64_t* count) {
  if (after < -1) return GBCC_ERR_INVALID_ARG;
  if (count) *count = gbcc::g_alloc_count.load();
  gbcc::g_fail_alloc_after.store(after);
  return GBCC_OK;
}
