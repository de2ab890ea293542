// Tensor-contraction engine of the CCSD residual.
//
// A residual is written as a fixed sequence of two operations on dense FP64
// device tensors addressed through index labels (the einstein notation of the
// reference's TiledArray expressions, one character per index):
//
//   assign(C("a,b,i,j"), beta, {coef * X("...") [* Y("...")], ...})
//   contract(C("a,b,i,j"), beta, alpha, A-terms("k,l,c,d"), B-terms("d,a,i,l"), class)
//
// The first pass over the program (PLAN) builds, for every call site, the
// offset tables that map labels to strides, chooses GEMM geometry and sizes
// the workspaces; later passes (EXEC) only launch kernels, so an EXEC pass can
// be captured into a CUDA graph.  Every contraction runs as
//   pack A, pack B (gather + linear combination, FP64 or split-BF16 slices)
//   -> GEMM (FP64 DFMA kernel or tcgen05 split-BF16 kernel)
//   -> scattered epilogue straight into C.
// Constant operands (integrals) are packed once per input set.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <stdexcept>
#include <functional>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/gbcc.h"
#include "kernels.h"

namespace gbcc {

struct Error : std::runtime_error {
  gbcc_status status;
  Error(gbcc_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define GBCC_CK(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      throw ::gbcc::Error(e_ == cudaErrorMemoryAllocation ? GBCC_ERR_OOM : GBCC_ERR_CUDA,  \
                          std::string(#call) + ": " + cudaGetErrorString(e_));           \
  } while (0)

void* dev_alloc(size_t bytes);
void dev_free(void* p);

struct Tensor {
  std::string name;
  double* d = nullptr;
  int rank = 0;
  int64_t dim[4] = {1, 1, 1, 1};
  bool constant = false;  // never written after the inputs are set
  int64_t size() const {
    int64_t n = 1;
    for (int k = 0; k < rank; ++k) n *= dim[k];
    return n;
  }
  int64_t stride(int k) const {
    int64_t s = 1;
    for (int q = rank - 1; q > k; --q) s *= dim[q];
    return s;
  }
};

// A tensor with index labels, e.g. Ix(G, "klcd").
struct Ix {
  const Tensor* t = nullptr;
  std::string lab;
};
inline Ix ix(const Tensor& t, const char* lab) { return Ix{&t, std::string(lab)}; }

// coef * a [* b]
struct Factor {
  double coef;
  Ix a;
  Ix b;  // b.t == nullptr: single factor
};
inline Factor f1(double c, const Ix& a) { return Factor{c, a, Ix{}}; }
inline Factor f2(double c, const Ix& a, const Ix& b) { return Factor{c, a, b}; }

// coef * x [* y]: a term of a contraction operand; a second factor y (its
// labels among the operand's) makes an outer-product term such as t1(d,i) t1(a,l)
struct Lin {
  double coef;
  Ix x;
  Ix y{};
};
inline Lin lin2(double c, const Ix& x, const Ix& y) { return Lin{c, x, y}; }

enum TermClass { kClassLadder = 0, kClassRing = 1, kClassOther = 2 };

enum class Mode { kPlan, kExec };

// index of a precision's plan in a call site: FP64 0, MIXED 1, FP64_TC 2
inline int plan_index(int precision) {
  return precision == GBCC_PREC_MIXED ? 1 : (precision == GBCC_PREC_FP64_TC ? 2 : 0);
}

struct DevTable {
  int64_t* d = nullptr;
  int64_t n = 0;
};

struct Site;  // per call site plan

struct SiteStat {
  double ms = 0.0;     // event time of the site's launches (profiling on)
  double gemm_ms = 0.0;  // of which the GEMM kernel
  double flops = 0.0;  // 2 M N K of a contraction, 0 for an assignment
  int pairs = 0;       // BF16 slice products on the tensor cores (0: FP64 / elementwise)
  int classes = 0;     // FP64_TC: launches, one per weight class (0 otherwise)
  int cls = -1;        // TermClass of a contraction, -1 for an assignment
  int64_t M = 0, N = 0, K = 0;  // GEMM shape (assignment: rows, columns, 0)
  int bn = 0;          // tensor cores: N tile width; -1: the short-K CUDA-core kernel
  int ksplit = 1;      // K split over CTAs
  int sps = 1;         // tensor cores: slices per pipeline stage
  int group = 1;       // tensor cores: M tiles per band of the tile order
};

struct OperandPlan;
struct GemmPlan;

// The process-wide autotune table: written as text by tune_save, merged from
// such a file by tune_load (false: unreadable or malformed, table unchanged)
bool tune_save(const std::string& path);
bool tune_load(const std::string& path);
void tune_clear();

class Engine {
 public:
  Engine();
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  void set_stream(cudaStream_t s) { stream_ = s; }
  cudaStream_t stream() const { return stream_; }
  void set_slices(int ladder, int ring, int other) {
    slices_[0] = ladder;
    slices_[1] = ring;
    slices_[2] = other;
  }
  void set_error_word(int* err) { err_ = err; }
  // at EXEC, use only the slice products of a split with this many slices
  // (0: all packed slices) for the contractions of each class
  void set_slice_limit(int ladder, int ring, int other) {
    slice_limit_[0] = ladder;
    slice_limit_[1] = ring;
    slice_limit_[2] = other;
  }
  // MMAs per TMEM accumulation, in (k-block, slice pair) steps, for
  // contractions with 3 slices and with fewer
  void set_chunk(int three_slices, int fewer) {
    chunk_ = three_slices;
    chunk_lo_ = fewer;
  }
  // Whether the next PLAN also builds the FP64-grade tensor-core plan
  // (GBCC_PREC_FP64_TC: fixed-point slices, one launch per weight class)
  void set_emulation(bool on) { emu_ = on; }
  bool emulation() const { return emu_; }
  // Record CUDA events around every operation of EXEC passes.
  void set_profile(bool on) { profile_ = on; }
  // Tensors a residual program reads but never writes (its amplitude inputs);
  // packs of them can be shared between contractions.
  void set_frozen(std::initializer_list<const Tensor*> ts) { frozen_ = std::unordered_set<const Tensor*>(ts); }
  std::vector<SiteStat> site_stats(int precision);

  // Persistent device tensor owned by the engine (allocated on first request).
  Tensor& tensor(const std::string& name, std::initializer_list<int64_t> dims, bool constant = false);
  Tensor* find(const std::string& name);
  // Give back a tensor's device storage (d becomes null; plans made while it
  // was allocated must not run again) and take it again, zeroed.
  void release(Tensor& t);
  void acquire(Tensor& t);

  // Program passes.  precision: GBCC_PREC_FP64 or GBCC_PREC_MIXED.
  void begin(Mode m, int precision);
  void end();
  bool planned() const { return planned_; }
  void reset_plans();  // inputs changed: rebuild everything on the next PLAN
  // After a PLAN pass: allocate the workspaces of every plan (once: EXEC
  // passes captured into graphs keep their pointers).
  void finalize();
  // Split packs of the constant operands of one tensor-core plan (MIXED or
  // FP64_TC), made once per PLAN; dedicated buffers, no workspace changes.
  void prepack(int precision);

  // C = beta*C + sum_t coef_t * a_t (* b_t); labels of each factor must be a
  // subset of C's labels (missing labels broadcast).
  void assign(const Ix& c, double beta, const std::vector<Factor>& terms);
  // C = beta*C + alpha * sum_K (sum_s a_s A_s)(sum_t b_t B_t)
  void contract(const Ix& c, double beta, double alpha, const std::vector<Lin>& A,
                const std::vector<Lin>& B, TermClass cls);
  // a fixed kernel sequence of the program, enqueued in program order at EXEC;
  // `launches` is the number of kernels it enqueues
  void custom(const std::function<void(cudaStream_t)>& fn, int launches);
  // time the candidate tile widths / K splits of every tensor-core contraction
  // of the finalised mixed plan on its operands and keep the fastest; a shape
  // already in the process's table (tune_load, or an earlier handle) takes
  // the stored choice untimed
  void autotune(int reps);

  // Statistics of the last EXEC pass (FLOPs of the contractions as planned).
  double flops() const { return flops_; }
  size_t device_bytes() const { return bytes_; }
  int gemm_tc_launches() const { return n_tc_; }
  // tensor-core GEMM launches since the engine was created (tuning included)
  int64_t gemm_tc_launches_total() const { return tc_total_; }
  int kernel_launches() const { return n_launch_; }

 private:
  Site& site();
  void prof_begin(Site& s);
  void prof_end(Site& s);
  void prof_gemm(Site& s);
  DevTable upload(const std::vector<int64_t>& v);
  __nv_bfloat16* tc_panel(OperandPlan& op, int side);
  void pack_panel(const OperandPlan& op, __nv_bfloat16* out);
  void launch_tc_classes(const GemmPlan& p, TermClass cls, __nv_bfloat16* const panel[2]);
  GemmTcArgs tc_args(const GemmPlan& p, TermClass cls, __nv_bfloat16* const panel[2]) const;
  void launch_tc(const GemmPlan& p, const GemmTcArgs& t);
  int slices_for(TermClass cls, double flops) const;

  cudaStream_t stream_ = nullptr;
  Mode mode_ = Mode::kPlan;
  int prec_ = GBCC_PREC_FP64;
  int slices_[3] = {3, 3, 3};
  int slice_limit_[3] = {0, 0, 0};
  size_t cursor_ = 0;
  bool planned_ = false;
  std::vector<std::unique_ptr<Site>> sites_;
  std::unordered_map<std::string, std::unique_ptr<Tensor>> tensors_;
  std::vector<void*> owned_;  // tables and constant-pack buffers
  // shared workspaces (sized during PLAN)
  size_t ws64_a_ = 0, ws64_b_ = 0, wsbf_a_ = 0, wsbf_b_ = 0, wspart_ = 0;
  double* wpart_ = nullptr;  // K-split partial tiles
  double* w64a_ = nullptr;
  double* w64b_ = nullptr;
  __nv_bfloat16* wbfa_ = nullptr;
  __nv_bfloat16* wbfb_ = nullptr;
  int* err_ = nullptr;
  // (k-block, slice pair) steps per TMEM accumulation of the tensor-core GEMM.
  // The tensor core's FP32 accumulation loses about an ulp of the running sum
  // per MMA, so 3-slice contractions (split error ~2^-24) accumulate 4 steps
  // at a time.  With 2 slices the split error (~2^-17) dominates even for 24
  // steps (measured: max error 4.67e-6 at 4 steps, 4.68e-6 at 24, K = 10240),
  // and the longer accumulations let the MMAs run further ahead of the
  // epilogue warps that drain them: 10240^3 at 2 slices 5.25 -> 4.79 ms.
  int chunk_ = 4;
  int chunk_lo_ = 24;
  bool profile_ = false;
  bool emu_ = false;
  bool packed_[3] = {false, false, false};
  std::unordered_set<const Tensor*> frozen_;
  std::unordered_map<std::string, std::vector<struct OperandPlan*>> pack_uses_;
  double flops_ = 0.0;
  size_t bytes_ = 0;
  int n_tc_ = 0;
  int64_t tc_total_ = 0;
  int n_launch_ = 0;
};

}  // namespace gbcc
