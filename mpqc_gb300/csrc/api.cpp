// C ABI of the CCSD amplitude solver (include/gbcc.h): handle, inputs,
// residual, energy and the Jacobi + DIIS solve loop.
//
// The solve loop follows CCSD::compute_ccsd (src/mpqc/chemistry/qc/lcao/cc/
// ccsd.h:331-477): t = 0 start with r1 = f_ai and r2 = g_abij, then per
// iteration error -> residual-augmented energy -> convergence test ->
// Jacobi update + DIIS extrapolation -> tau -> R1 -> R2.
#include <array>
#include <chrono>
#include <cmath>
#include <limits>
#include <utility>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbcc.h"
#include "triples.h"
#include "../../include/gbcc_testing.h"
#include "ccsd_program.h"
#include "engine.h"
#include "kernels.h"

using gbcc::Error;

struct gbcc_handle {
  gbcc_config cfg{};
  std::string last_error;
  cudaStream_t stream = nullptr;
  std::unique_ptr<gbcc::Engine> eng;
  std::unique_ptr<gbcc::Engine> aux;  // one-off setup operations
  gbcc::CcsdTensors S{};
  bool inputs_set = false;
  bool tensors_incomplete = false;  // an allocation failed inside create_tensors
  int* d_err = nullptr;
  double* d_partial = nullptr;  // reduction scratch [kReduceBlocks * 16]
  double* d_out = nullptr;      // reduction results
  double* h_out = nullptr;      // pinned mirror
  // DIIS storage (allocated on the first solve)
  double *x1 = nullptr, *x2 = nullptr, *e1 = nullptr, *e2 = nullptr;
  double *Bmat = nullptr, *coef = nullptr;
  int* d_nskip = nullptr;
  int ndiis_alloc = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int last_launches = 0;  // kernels launched by the last residual
  cudaEvent_t slots[8] = {};
  std::vector<double> prof_gemm_ms;
  std::vector<std::array<int64_t, 3>> prof_dims;
  std::vector<std::array<int32_t, 4>> prof_tiles;
  // residual program captured as a CUDA graph, one per precision (FP64,
  // mixed, FP64_TC: gbcc::plan_index)
  cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
  int graph_launches[3] = {0, 0, 0};
  bool profiling = false;
  bool calibrating = false;
  // slice counts in use per class (ladder, ring, other) and, for classes the
  // calibration chose, the measured relative residual change; -1 when not measured
  int slices_used[3] = {3, 3, 3};
  double slice_err[3] = {-1.0, -1.0, -1.0};
  // amplitudes seeding the next solve (gbcc_set_amplitudes / load), and
  // whether t1/t2 hold the result of the last solve (gbcc_save_amplitudes)
  double *seed1 = nullptr, *seed2 = nullptr;
  bool seeded = false;
  bool have_solution = false;
  double last_e = 0.0;
  // whole-solve graph (use_graphs = 2): the residual programs as graphs (the
  // FP64-grade precision, mixed), the instantiated loop, its device state,
  // history and timestamps
  cudaGraph_t rgraph[2] = {nullptr, nullptr};
  cudaGraphExec_t solve_exec = nullptr;
  gbcc::SolveState* d_state = nullptr;
  double* d_history = nullptr;
  unsigned long long* d_stamps = nullptr;
};

namespace {

thread_local std::string g_create_error;

int64_t n1_of(const gbcc_handle* h) { return h->cfg.v * h->cfg.o; }
int64_t n2_of(const gbcc_handle* h) { return h->cfg.v * h->cfg.v * h->cfg.o * h->cfg.o; }

gbcc_status fail(gbcc_handle* h, gbcc_status s, const std::string& msg) {
  if (h) h->last_error = msg;
  return s;
}

template <class F>
gbcc_status guarded(gbcc_handle* h, F&& f) {
  if (!h) return GBCC_ERR_INVALID_ARG;
  if (h->tensors_incomplete)
    return fail(h, GBCC_ERR_STATE, "an allocation failure left the handle's tensors incomplete: destroy it");
  try {
    if (cudaSetDevice(h->cfg.device) != cudaSuccess)
      throw Error(GBCC_ERR_CUDA, "cudaSetDevice failed");
    gbcc_status s = f();
    if (s == GBCC_OK || s == GBCC_ERR_NOT_CONVERGED) h->last_error.clear();
    return s;
  } catch (const Error& e) {
    cudaGetLastError();
    return fail(h, e.status, e.what());
  } catch (const std::bad_alloc&) {
    return fail(h, GBCC_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(h, GBCC_ERR_CUDA, e.what());
  }
}

// The handle's tensors, on the first input call.  An allocation failure part
// way leaves them incomplete: the handle then refuses every call but
// gbcc_destroy (GBCC_ERR_STATE).
void create_tensors(gbcc_handle* h, int64_t naux, int64_t nao) {
  if (h->S.t1) return;
  try {
    h->S.create(*h->eng, h->cfg.o, h->cfg.v, naux, nao);
  } catch (...) {
    h->tensors_incomplete = true;
    throw;
  }
}

void copy_in(double* dst, const double* src, int64_t n, cudaStream_t st) {
  GBCC_CK(cudaMemcpyAsync(dst, src, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDefault, st));
}

void copy_out(double* dst, const double* src, int64_t n, cudaStream_t st) {
  GBCC_CK(cudaMemcpyAsync(dst, src, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDefault, st));
}

// Device-to-host read on the handle's own stream (not the legacy default
// stream, which would serialise concurrent solves of other handles).
void read_back(gbcc_handle* h, void* dst, const void* src, size_t bytes) {
  GBCC_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
  GBCC_CK(cudaStreamSynchronize(h->stream));
}

// Check the device error word and any pending CUDA error after a sync.
void sync_check(gbcc_handle* h) {
  GBCC_CK(cudaStreamSynchronize(h->stream));
  GBCC_CK(cudaGetLastError());
  int err = 0;
  read_back(h, &err, h->d_err, sizeof(int));
  if (err != gbcc::kDevOk) {
    GBCC_CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    GBCC_CK(cudaStreamSynchronize(h->stream));
    throw Error(GBCC_ERR_TIMEOUT, "a bounded device-side wait gave up (tensor-core pipeline)");
  }
}

bool check_config(const gbcc_config* c, std::string& why) {
  if (c->o < 1 || c->v < 1) { why = "o and v must be >= 1"; return false; }
  if (c->o > 4096 || c->v > 8192) { why = "o or v out of range"; return false; }
  if (c->precision != GBCC_PREC_FP64 && c->precision != GBCC_PREC_MIXED && c->precision != GBCC_PREC_FP64_TC) {
    why = "bad precision";
    return false;
  }
  if (c->refine_precision != GBCC_PREC_FP64 && c->refine_precision != GBCC_PREC_FP64_TC) {
    why = "refine_precision must be GBCC_PREC_FP64 or GBCC_PREC_FP64_TC";
    return false;
  }
  for (int s : {c->slices_ladder, c->slices_ring, c->slices_other})
    if (s < 0 || s > 3) { why = "slices must be 0 (automatic) or 1..3"; return false; }
  if (!(c->slice_tolerance > 0.0)) { why = "slice_tolerance must be > 0"; return false; }
  if (c->n_diis < 1 || c->n_diis > 16) { why = "n_diis must be 1..16"; return false; }
  if (c->diis_ngroup < 1 || c->diis_start < 0 || c->diis_group_nstart < 0) { why = "bad DIIS parameters"; return false; }
  if (!(c->diis_damp >= 0.0)) { why = "diis_damp must be >= 0"; return false; }
  if (c->max_iter < 1) { why = "max_iter must be >= 1"; return false; }
  if (!(c->target_precision > 0.0)) { why = "target_precision must be > 0"; return false; }
  if (c->refine_iters < 0) { why = "refine_iters must be >= 0"; return false; }
  if (!(c->mixed_switch_precision >= 0.0)) { why = "mixed_switch_precision must be >= 0"; return false; }
  if (c->refine_reset_diis != 0 && c->refine_reset_diis != 1) { why = "refine_reset_diis must be 0 or 1"; return false; }
  if (c->use_graphs < 0 || c->use_graphs > 2) { why = "use_graphs must be 0, 1 or 2"; return false; }
  return true;
}

void drop_graphs(gbcc_handle* h) {
  for (auto& g : h->graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  for (auto& g : h->rgraph) {
    if (g) cudaGraphDestroy(g);
    g = nullptr;
  }
  if (h->solve_exec) cudaGraphExecDestroy(h->solve_exec);
  h->solve_exec = nullptr;
  for (int& n : h->graph_launches) n = 0;
}

// The FP64-grade precision of a handle: its own for FP64 and FP64_TC handles,
// the refinement's for mixed ones.
int hi_prec(const gbcc_handle* h) {
  return h->cfg.precision == GBCC_PREC_MIXED ? h->cfg.refine_precision : h->cfg.precision;
}

// whether the handle's plan includes the FP64_TC contractions
bool uses_fp64_tc(const gbcc_handle* h) { return hi_prec(h) == GBCC_PREC_FP64_TC; }

// r1, r2 of the device-resident t1, t2, tau.  The first evaluation in each
// precision is captured into a CUDA graph (every launch of the EXEC pass has
// fixed pointers, sizes and tensor maps once the plan is finalised); later
// evaluations replay it.  Returns the number of kernels it enqueued.
int enqueue_residual_program(gbcc_handle* h, int precision) {
  h->eng->prepack(precision);  // once per plan; no workspace changes
  auto direct = [&]() {
    h->eng->begin(gbcc::Mode::kExec, precision);
    gbcc::residual_program(*h->eng, h->S);
    h->eng->end();
    return h->eng->kernel_launches();
  };
  if (!h->cfg.use_graphs || h->profiling || h->calibrating) return direct();
  const int gi = gbcc::plan_index(precision);
  if (!h->graph[gi]) {
    cudaGraph_t g = nullptr;
    GBCC_CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int n = 0;
    try {
      n = direct();
    } catch (...) {
      cudaStreamEndCapture(h->stream, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      throw;
    }
    GBCC_CK(cudaStreamEndCapture(h->stream, &g));
    cudaGraphExec_t ge = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) throw Error(GBCC_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    h->graph[gi] = ge;
    h->graph_launches[gi] = n;
  }
  GBCC_CK(cudaGraphLaunch(h->graph[gi], h->stream));
  return h->graph_launches[gi];
}

void run_residual(gbcc_handle* h, int precision) {
  gbcc::launch_make_tau(h->cfg.o, h->cfg.v, h->S.t1->d, h->S.t2->d, h->S.tau->d, h->stream);
  h->last_launches = 1 + enqueue_residual_program(h, precision);
}

// E and error of the current t/tau/r (device-resident); returns {E, error}
std::pair<double, double> energy_error(gbcc_handle* h) {
  gbcc::launch_energy_terms(h->cfg.o, h->cfg.v, h->S.r1->d, h->S.r2->d, h->S.f_ai->d, h->S.g_abij->d,
                            h->S.t1->d, h->S.tau->d, h->d_partial, h->d_out, h->stream);
  GBCC_CK(cudaMemcpyAsync(h->h_out, h->d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  sync_check(h);
  const double* s = h->h_out;
  const double E = 2.0 * s[2] + s[3];
  const double err = std::sqrt(s[0] + s[1]) / static_cast<double>(n1_of(h) + n2_of(h));
  return {E, err};
}

void ensure_diis(gbcc_handle* h) {
  const int nd = h->cfg.n_diis;
  if (h->ndiis_alloc == nd) return;
  for (void* p : {(void*)h->x1, (void*)h->x2, (void*)h->e1, (void*)h->e2, (void*)h->Bmat,
                  (void*)h->coef, (void*)h->d_nskip})
    gbcc::dev_free(p);
  const size_t n1 = static_cast<size_t>(n1_of(h)), n2 = static_cast<size_t>(n2_of(h));
  h->x1 = static_cast<double*>(gbcc::dev_alloc(nd * n1 * sizeof(double)));
  h->e1 = static_cast<double*>(gbcc::dev_alloc(nd * n1 * sizeof(double)));
  h->x2 = static_cast<double*>(gbcc::dev_alloc(nd * n2 * sizeof(double)));
  h->e2 = static_cast<double*>(gbcc::dev_alloc(nd * n2 * sizeof(double)));
  h->Bmat = static_cast<double*>(gbcc::dev_alloc(nd * nd * sizeof(double)));
  h->coef = static_cast<double*>(gbcc::dev_alloc(nd * sizeof(double)));
  h->d_nskip = static_cast<int*>(gbcc::dev_alloc(sizeof(int)));
  h->ndiis_alloc = nd;
}

// The residual program of one precision as a (not instantiated) graph.
cudaGraph_t capture_residual_graph(gbcc_handle* h, int precision) {
  h->eng->prepack(precision);
  cudaGraph_t g = nullptr;
  GBCC_CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  try {
    h->eng->begin(gbcc::Mode::kExec, precision);
    gbcc::residual_program(*h->eng, h->S);
    h->eng->end();
  } catch (...) {
    cudaStreamEndCapture(h->stream, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    throw;
  }
  GBCC_CK(cudaStreamEndCapture(h->stream, &g));
  return g;
}

// Capture what fn enqueues on the handle's stream into the (empty) graph g.
template <class F>
void capture_into(gbcc_handle* h, cudaGraph_t g, F&& fn) {
  GBCC_CK(cudaStreamBeginCaptureToGraph(h->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  cudaGraph_t out = nullptr;
  try {
    fn();
  } catch (...) {
    cudaStreamEndCapture(h->stream, &out);
    cudaGetLastError();
    throw;
  }
  GBCC_CK(cudaStreamEndCapture(h->stream, &out));
}

// the node of g that no other node depends on (g has exactly one)
cudaGraphNode_t sink_node(cudaGraph_t g) {
  size_t n = 0;
  GBCC_CK(cudaGraphGetNodes(g, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  GBCC_CK(cudaGraphGetNodes(g, nodes.data(), &n));
  cudaGraphNode_t sink = nullptr;
  for (cudaGraphNode_t nd : nodes) {
    size_t k = 0;
    GBCC_CK(cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &k));
    if (k == 0) {
      if (sink) throw Error(GBCC_ERR_CUDA, "solve graph: captured segment has more than one sink");
      sink = nd;
    }
  }
  if (!sink) throw Error(GBCC_ERR_CUDA, "solve graph: empty captured segment");
  return sink;
}

// A conditional node of type `type` after `dep` in graph g; returns its body.
cudaGraph_t add_conditional(cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraphConditionalHandle hc,
                            cudaGraphConditionalNodeType type, cudaGraphNode_t* node) {
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = hc;
  p.conditional.type = type;
  p.conditional.size = 1;
  GBCC_CK(cudaGraphAddNode(node, g, dep, nullptr, dep ? 1 : 0, &p));
  return p.conditional.phGraph_out[0];
}

// The whole solve loop as one graph (use_graphs = 2): a WHILE node whose body
// is one iteration -- energy terms, the decision kernel (solve_graph.cu), the
// Jacobi + DIIS update and the residual of the precision it chose -- so the
// host launches the graph once per solve and synchronises once.
void build_solve_graph(gbcc_handle* h) {
  const gbcc_config& c = h->cfg;
  const bool mixed = c.precision == GBCC_PREC_MIXED;
  cudaStream_t st = h->stream;
  if (!h->rgraph[0]) h->rgraph[0] = capture_residual_graph(h, hi_prec(h));
  if (mixed && !h->rgraph[1]) h->rgraph[1] = capture_residual_graph(h, GBCC_PREC_MIXED);
  if (!h->d_state) h->d_state = static_cast<gbcc::SolveState*>(gbcc::dev_alloc(sizeof(gbcc::SolveState)));
  if (!h->d_history) h->d_history = static_cast<double*>(gbcc::dev_alloc((c.max_iter + 1) * 3 * sizeof(double)));
  if (!h->d_stamps)
    h->d_stamps = static_cast<unsigned long long*>(gbcc::dev_alloc((c.max_iter + 1) * 2 * sizeof(unsigned long long)));
  cudaGraph_t G = nullptr;
  GBCC_CK(cudaGraphCreate(&G, 0));
  struct GraphGuard {
    cudaGraph_t g;
    ~GraphGuard() {
      if (g) cudaGraphDestroy(g);
    }
  } guard{G};
  cudaGraphConditionalHandle hloop, hup, hmix, hf64;
  GBCC_CK(cudaGraphConditionalHandleCreate(&hloop, G, 1, cudaGraphCondAssignDefault));
  cudaGraphNode_t wnode;
  cudaGraph_t body = add_conditional(G, nullptr, hloop, cudaGraphCondTypeWhile, &wnode);
  GBCC_CK(cudaGraphConditionalHandleCreate(&hup, body, 0, cudaGraphCondAssignDefault));
  GBCC_CK(cudaGraphConditionalHandleCreate(&hmix, body, 0, cudaGraphCondAssignDefault));
  GBCC_CK(cudaGraphConditionalHandleCreate(&hf64, body, 0, cudaGraphCondAssignDefault));
  gbcc::CcsdTensors& S = h->S;
  gbcc::SolveParams p{};
  p.n1 = n1_of(h);
  p.n2 = n2_of(h);
  p.max_iter = c.max_iter;
  p.n_diis = c.n_diis;
  p.diis_start = c.diis_start;
  p.diis_ngroup = c.diis_ngroup;
  p.diis_group_nstart = c.diis_group_nstart;
  p.refine_iters = c.refine_iters;
  p.reset_diis = c.refine_reset_diis;
  p.target = c.target_precision;
  p.switch_precision = c.mixed_switch_precision;
  p.Bmat = h->Bmat;
  p.sums = h->d_out;
  p.state = h->d_state;
  p.history = h->d_history;
  p.cond_loop = hloop;
  p.cond_update = hup;
  p.cond_mixed = hmix;
  p.cond_fp64 = hf64;
  capture_into(h, body, [&] {
    gbcc::launch_energy_terms(c.o, c.v, S.r1->d, S.r2->d, S.f_ai->d, S.g_abij->d, S.t1->d, S.tau->d, h->d_partial,
                              h->d_out, st);
    gbcc::launch_solve_decide(p, st);
  });
  cudaGraphNode_t decide = sink_node(body);
  cudaGraphNode_t nup;
  cudaGraph_t ub = add_conditional(body, &decide, hup, cudaGraphCondTypeIf, &nup);
  gbcc::DiisArgs d{};
  d.dyn = &h->d_state->diis;
  d.o = c.o;
  d.v = c.v;
  d.eps_o = S.eps_o->d;
  d.eps_v = S.eps_v->d;
  d.dinv1 = S.Dinv1->d;
  d.dinv2 = S.Dinv2->d;
  d.t1 = S.t1->d;
  d.t2 = S.t2->d;
  d.r1 = S.r1->d;
  d.r2 = S.r2->d;
  d.x1 = h->x1;
  d.x2 = h->x2;
  d.e1 = h->e1;
  d.e2 = h->e2;
  d.ndiis = c.n_diis;
  d.partial = h->d_partial;
  d.Bmat = h->Bmat;
  d.coef = h->coef;
  d.damping = c.diis_damp;
  d.nskip_out = h->d_nskip;
  capture_into(h, ub, [&] {
    gbcc::launch_diis_step(d, st);
    gbcc::launch_diis_extrapolate(c.o, c.v, h->x1, h->x2, h->coef, c.n_diis, nullptr, 0, S.t1->d, S.t2->d,
                                  S.tau->d, st, &h->d_state->diis);
  });
  // residual of the chosen precision, timestamped on the device
  auto add_residual = [&](cudaGraphConditionalHandle hc, cudaGraphNode_t dep, cudaGraph_t rg) {
    cudaGraphNode_t n, s0, child, s1;
    cudaGraph_t rb = add_conditional(body, &dep, hc, cudaGraphCondTypeIf, &n);
    if (!rg) {
      GBCC_CK(cudaGraphAddEmptyNode(&s0, rb, nullptr, 0));
      return n;
    }
    GBCC_CK(gbcc::add_stamp_node(rb, nullptr, 0, h->d_stamps, h->d_state, 0, &s0));
    GBCC_CK(cudaGraphAddChildGraphNode(&child, rb, &s0, 1, rg));
    GBCC_CK(gbcc::add_stamp_node(rb, &child, 1, h->d_stamps, h->d_state, 1, &s1));
    return n;
  };
  cudaGraphNode_t last = add_residual(hf64, nup, h->rgraph[0]);
  add_residual(hmix, last, mixed ? h->rgraph[1] : nullptr);
  cudaGraphExec_t ge = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&ge, G, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(GBCC_ERR_CUDA, std::string("solve graph instantiation: ") + cudaGetErrorString(e));
  }
  h->solve_exec = ge;
}

void print_iter(int iter, double dE, double error, double E, double t) {
  if (iter == 1)
    std::printf("%3s \t %10s \t %10s \t %15s \t %10s \n", "iter", "deltaE", "residual", "energy",
                "total time/s");
  std::printf("%3i \t %10.5e \t %10.5e \t %15.12f \t %10.1f \n", iter, dE, error, E, t);
  std::fflush(stdout);
}

void validate_eps(const double* eps_o, const double* eps_v, int64_t o, int64_t v) {
  std::vector<double> eo(o), ev(v);
  GBCC_CK(cudaMemcpy(eo.data(), eps_o, o * sizeof(double), cudaMemcpyDefault));
  GBCC_CK(cudaMemcpy(ev.data(), eps_v, v * sizeof(double), cudaMemcpyDefault));
  for (int64_t i = 0; i < o; ++i)
    for (int64_t a = 0; a < v; ++a)
      if (!std::isfinite(eo[i]) || !std::isfinite(ev[a]) || eo[i] - ev[a] == 0.0)
        throw Error(GBCC_ERR_INVALID_ARG,
                    "orbital energies non-finite or degenerate across the gap (zero Jacobi denominator)");
}

// max|a - ref| / max|ref| over n device doubles
double rel_change(gbcc_handle* h, int64_t n, const double* a, const double* ref) {
  auto* out = reinterpret_cast<unsigned long long*>(h->d_out + 8);
  GBCC_CK(cudaMemsetAsync(out, 0, 2 * sizeof(double), h->stream));
  gbcc::launch_maxabs_diff(n, a, ref, out, h->stream);
  GBCC_CK(cudaMemcpyAsync(h->h_out + 8, h->d_out + 8, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  sync_check(h);
  const double md = h->h_out[8], mb = h->h_out[9];
  if (mb == 0.0) return md == 0.0 ? 0.0 : std::numeric_limits<double>::infinity();
  return md / mb;
}

// Tile widths and K splits of the mixed plan from timing (config autotune)
void tune_plan(gbcc_handle* h) {
  if (h->cfg.precision != GBCC_PREC_MIXED || !h->cfg.autotune) return;
  drop_graphs(h);
  h->eng->autotune(3);
  sync_check(h);
}

// The particle-particle ladder runs over a <= b, i <= j: amplitudes must be
// pair-symmetric, t2(a,b,i,j) = t2(b,a,j,i) (closed-shell CCSD amplitudes are)
void check_pair_symmetric(gbcc_handle* h) {
  auto* out = reinterpret_cast<unsigned long long*>(h->d_out + 8);
  GBCC_CK(cudaMemsetAsync(out, 0, 2 * sizeof(double), h->stream));
  gbcc::launch_pair_asym(h->cfg.o, h->cfg.v, h->S.t2->d, out, h->stream);
  GBCC_CK(cudaMemcpyAsync(h->h_out + 8, h->d_out + 8, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  sync_check(h);
  if (!(h->h_out[8] <= 1e-12 * h->h_out[9]))
    throw Error(GBCC_ERR_INVALID_ARG, "t2 is not pair-symmetric (t2(a,b,i,j) != t2(b,a,j,i)): max difference " +
                                          std::to_string(h->h_out[8]) + " of max |t2| " + std::to_string(h->h_out[9]));
}

void plan_residual(gbcc_handle* h) {
  drop_graphs(h);
  h->eng->reset_plans();
  h->eng->set_slices(h->slices_used[0], h->slices_used[1], h->slices_used[2]);
  h->eng->set_frozen({h->S.t1, h->S.t2, h->S.tau});
  h->eng->set_emulation(uses_fp64_tc(h));
  h->eng->begin(gbcc::Mode::kPlan, GBCC_PREC_FP64);
  gbcc::residual_program(*h->eng, h->S);
  h->eng->end();
  // workspaces, then the split packs of the constant operands for the
  // tensor-core precisions the handle runs (others are packed on first use)
  h->eng->finalize();
  if (h->cfg.precision == GBCC_PREC_MIXED) h->eng->prepack(GBCC_PREC_MIXED);
  if (uses_fp64_tc(h)) h->eng->prepack(GBCC_PREC_FP64_TC);
}

// Slice counts for the classes configured as 0 (automatic), chosen from their
// measured error.  The residual at the calibration amplitudes with every
// automatic class at 3 slices is the reference; each automatic class in turn
// is evaluated with 2, then 1 slices (the other classes at 3) and keeps the
// smallest count whose max|dr| / max|r|, over r1 and r2, is at most
// slice_tolerance.  The amplitudes are the caller's (t1_in, t2_in: host or
// device) or, when those are NULL, probe amplitudes: two Jacobi steps from
// t = 0 (MP2 amplitudes, then one residual further, so t1 is nonzero).
// The residual plan is rebuilt for the chosen counts; t1 = t2 = tau = 0 after.
void calibrate_slices(gbcc_handle* h, const double* t1_in, const double* t2_in) {
  gbcc::CcsdTensors& S = h->S;
  const int req[3] = {h->cfg.slices_ladder, h->cfg.slices_ring, h->cfg.slices_other};
  const int64_t o = h->cfg.o, v = h->cfg.v, n1 = n1_of(h), n2 = n2_of(h);
  cudaStream_t st = h->stream;
  for (int k = 0; k < 3; ++k) {
    h->slices_used[k] = req[k] == 0 ? 3 : req[k];
    h->slice_err[k] = -1.0;
  }
  plan_residual(h);
  struct Guard {
    gbcc_handle* h;
    double* ref = nullptr;
    ~Guard() {
      h->calibrating = false;
      h->eng->set_slice_limit(0, 0, 0);
      gbcc::dev_free(ref);
    }
  } guard{h};
  h->calibrating = true;
  if (t1_in && t2_in) {
    GBCC_CK(cudaMemcpyAsync(S.t1->d, t1_in, n1 * sizeof(double), cudaMemcpyDefault, st));
    GBCC_CK(cudaMemcpyAsync(S.t2->d, t2_in, n2 * sizeof(double), cudaMemcpyDefault, st));
    check_pair_symmetric(h);
  } else {
    GBCC_CK(cudaMemsetAsync(S.t1->d, 0, n1 * sizeof(double), st));
    GBCC_CK(cudaMemsetAsync(S.t2->d, 0, n2 * sizeof(double), st));
    gbcc::launch_jacobi_inplace(o, v, S.eps_o->d, S.eps_v->d, S.f_ai->d, S.g_abij->d, S.t1->d, S.t2->d, st);
    gbcc::launch_make_tau(o, v, S.t1->d, S.t2->d, S.tau->d, st);
    enqueue_residual_program(h, GBCC_PREC_MIXED);
    gbcc::launch_jacobi_inplace(o, v, S.eps_o->d, S.eps_v->d, S.r1->d, S.r2->d, S.t1->d, S.t2->d, st);
  }
  gbcc::launch_make_tau(o, v, S.t1->d, S.t2->d, S.tau->d, st);
  enqueue_residual_program(h, GBCC_PREC_MIXED);
  guard.ref = static_cast<double*>(gbcc::dev_alloc((n1 + n2) * sizeof(double)));
  GBCC_CK(cudaMemcpyAsync(guard.ref, S.r1->d, n1 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  GBCC_CK(cudaMemcpyAsync(guard.ref + n1, S.r2->d, n2 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  for (int k = 0; k < 3; ++k) {
    if (req[k] != 0) continue;
    h->slice_err[k] = 0.0;
    for (int s = 2; s >= 1; --s) {
      int lim[3] = {0, 0, 0};
      lim[k] = s;
      h->eng->set_slice_limit(lim[0], lim[1], lim[2]);
      enqueue_residual_program(h, GBCC_PREC_MIXED);
      const double e = std::max(rel_change(h, n1, S.r1->d, guard.ref), rel_change(h, n2, S.r2->d, guard.ref + n1));
      if (!(e <= h->cfg.slice_tolerance)) break;
      h->slices_used[k] = s;
      h->slice_err[k] = e;
    }
  }
  h->eng->set_slice_limit(0, 0, 0);
  GBCC_CK(cudaMemsetAsync(S.t1->d, 0, n1 * sizeof(double), st));
  GBCC_CK(cudaMemsetAsync(S.t2->d, 0, n2 * sizeof(double), st));
  GBCC_CK(cudaMemsetAsync(S.tau->d, 0, n2 * sizeof(double), st));
  sync_check(h);
  h->calibrating = false;
  if (h->slices_used[0] != 3 || h->slices_used[1] != 3 || h->slices_used[2] != 3) plan_residual(h);
  sync_check(h);
  tune_plan(h);
}

// Derived constants, the residual plan for both precisions and (mixed
// handles) the split copies of the constant operands.
void commit_inputs(gbcc_handle* h) {
  gbcc::CcsdTensors& S = h->S;
  h->aux->reset_plans();
  h->aux->begin(gbcc::Mode::kPlan, GBCC_PREC_FP64);
  gbcc::setup_program(*h->aux, S);
  h->aux->end();
  h->aux->finalize();
  h->aux->begin(gbcc::Mode::kExec, GBCC_PREC_FP64);
  gbcc::setup_program(*h->aux, S);
  h->aux->end();
  // (ab|cd) is read only by the set-up (its pair-symmetric G+/G- copies feed
  // the ladder): its v^4 storage is given back until inputs are set again
  if (S.Gabcd) h->eng->release(*S.Gabcd);
  const int req[3] = {h->cfg.slices_ladder, h->cfg.slices_ring, h->cfg.slices_other};
  if (h->cfg.precision == GBCC_PREC_MIXED && (req[0] == 0 || req[1] == 0 || req[2] == 0)) {
    calibrate_slices(h, nullptr, nullptr);
  } else {
    for (int k = 0; k < 3; ++k) {
      h->slices_used[k] = req[k] == 0 ? 3 : req[k];
      h->slice_err[k] = -1.0;
    }
    plan_residual(h);
    sync_check(h);
    tune_plan(h);
  }
  h->inputs_set = true;
}

}  // namespace

// Thread-local message read by gbcc_last_error(NULL) (handle-free entry points).
void gbcc_set_thread_error(const std::string& msg) { g_create_error = msg; }

// Dimensions and device of a handle, for the SCF input producer (scf.cpp).
bool gbcc_internal_dims(const gbcc_handle* h, int64_t* o, int64_t* v, int* device) {
  if (!h) return false;
  *o = h->cfg.o;
  *v = h->cfg.v;
  *device = h->cfg.device;
  return true;
}

extern "C" {

int gbcc_abi_version(void) { return GBCC_ABI_VERSION; }

const char* gbcc_status_string(gbcc_status s) {
  switch (s) {
    case GBCC_OK: return "ok";
    case GBCC_ERR_INVALID_ARG: return "invalid argument";
    case GBCC_ERR_OOM: return "out of device memory";
    case GBCC_ERR_CUDA: return "CUDA error";
    case GBCC_ERR_NOT_CONVERGED: return "not converged";
    case GBCC_ERR_TIMEOUT: return "device wait timed out";
    case GBCC_ERR_STATE: return "call out of order";
    case GBCC_ERR_NUMERIC: return "non-finite value";
  }
  return "unknown status";
}

void gbcc_config_default(gbcc_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->precision = GBCC_PREC_FP64;
  c->slices_ladder = 0;
  c->slices_ring = 0;
  c->slices_other = 0;
  c->refine_iters = 2;
  c->refine_precision = GBCC_PREC_FP64;
  c->mixed_switch_precision = 0.0;
  c->max_iter = 30;
  c->target_precision = 1e-9;
  c->diis_start = 1;
  c->n_diis = 8;
  c->diis_damp = 0.0;
  c->diis_ngroup = 1;
  c->diis_group_nstart = 1;
  c->verbose = 0;
  c->device = 0;
  c->use_graphs = 2;
  c->slice_tolerance = 1e-5;
  c->autotune = 1;
  c->refine_reset_diis = 1;
}

gbcc_status gbcc_create(gbcc_handle** out, const gbcc_config* cfg) {
  g_create_error.clear();
  if (!out || !cfg) {
    g_create_error = "gbcc_create: NULL argument";
    return GBCC_ERR_INVALID_ARG;
  }
  *out = nullptr;
  std::string why;
  if (!check_config(cfg, why)) {
    g_create_error = "gbcc_create: " + why;
    return GBCC_ERR_INVALID_ARG;
  }
  auto h = std::make_unique<gbcc_handle>();
  h->cfg = *cfg;
  try {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      throw Error(GBCC_ERR_CUDA, "no CUDA device available");
    }
    if (cfg->device < 0 || cfg->device >= ndev) throw Error(GBCC_ERR_INVALID_ARG, "bad device ordinal");
    GBCC_CK(cudaSetDevice(cfg->device));
    GBCC_CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    GBCC_CK(cudaEventCreate(&h->ev0));
    GBCC_CK(cudaEventCreate(&h->ev1));
    h->eng = std::make_unique<gbcc::Engine>();
    h->aux = std::make_unique<gbcc::Engine>();
    h->eng->set_stream(h->stream);
    h->aux->set_stream(h->stream);
    h->eng->set_slices(cfg->slices_ladder, cfg->slices_ring, cfg->slices_other);
    h->d_err = static_cast<int*>(gbcc::dev_alloc(sizeof(int)));
    GBCC_CK(cudaMemset(h->d_err, 0, sizeof(int)));
    h->eng->set_error_word(h->d_err);
    h->d_partial = static_cast<double*>(gbcc::dev_alloc(gbcc::kReduceBlocks * 16 * sizeof(double)));
    h->d_out = static_cast<double*>(gbcc::dev_alloc(16 * sizeof(double)));
    GBCC_CK(cudaMallocHost(&h->h_out, 16 * sizeof(double)));
  } catch (const Error& e) {
    g_create_error = e.what();
    if (h->h_out) cudaFreeHost(h->h_out);
    gbcc::dev_free(h->d_err);
    gbcc::dev_free(h->d_partial);
    gbcc::dev_free(h->d_out);
    return e.status;
  }
  *out = h.release();
  return GBCC_OK;
}

gbcc_status gbcc_set_inputs(gbcc_handle* h, const gbcc_inputs* in) {
  return guarded(h, [&]() -> gbcc_status {
    if (!in) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_inputs: NULL inputs");
    const double* ptrs[] = {in->eps_o, in->eps_v, in->Fia, in->Fij, in->Fab, in->Gijab,
                            in->Gijkl, in->Giajb, in->Gijka, in->Giabc, in->Gabcd};
    for (const double* p : ptrs)
      if (!p) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_inputs: NULL input array");
    const int64_t o = h->cfg.o, v = h->cfg.v;
    validate_eps(in->eps_o, in->eps_v, o, v);
    create_tensors(h, 0, 0);
    if (h->S.naux > 0 || h->S.nao > 0)
      throw Error(GBCC_ERR_STATE, "gbcc_set_inputs: the handle holds density-fitted or integral-direct inputs");
    gbcc::CcsdTensors& S = h->S;
    h->inputs_set = false;
    h->have_solution = false;
    h->seeded = false;
    copy_in(S.eps_o->d, in->eps_o, o, h->stream);
    copy_in(S.eps_v->d, in->eps_v, v, h->stream);
    copy_in(S.Fia->d, in->Fia, o * v, h->stream);
    copy_in(S.Fij->d, in->Fij, o * o, h->stream);
    copy_in(S.Fab->d, in->Fab, v * v, h->stream);
    copy_in(S.Gijab->d, in->Gijab, o * o * v * v, h->stream);
    copy_in(S.Gijkl->d, in->Gijkl, o * o * o * o, h->stream);
    copy_in(S.Giajb->d, in->Giajb, o * v * o * v, h->stream);
    copy_in(S.Gijka->d, in->Gijka, o * o * o * v, h->stream);
    copy_in(S.Giabc->d, in->Giabc, o * v * v * v, h->stream);
    h->eng->acquire(*S.Gabcd);
    copy_in(S.Gabcd->d, in->Gabcd, v * v * v * v, h->stream);
    commit_inputs(h);
    return GBCC_OK;
  });
}

gbcc_status gbcc_set_df_inputs(gbcc_handle* h, const gbcc_df_inputs* in) {
  return guarded(h, [&]() -> gbcc_status {
    if (!in) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_df_inputs: NULL inputs");
    const double* ptrs[] = {in->eps_o, in->eps_v, in->Fia, in->Fij, in->Fab, in->Gijab,
                            in->Gijkl, in->Giajb, in->Gijka, in->Xai, in->Xab};
    for (const double* p : ptrs)
      if (!p) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_df_inputs: NULL input array");
    if (in->naux < 1 || in->naux > (int64_t{1} << 20))
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_df_inputs: naux out of range");
    const int64_t o = h->cfg.o, v = h->cfg.v, nq = in->naux;
    validate_eps(in->eps_o, in->eps_v, o, v);
    create_tensors(h, nq, 0);
    if (h->S.nao > 0) throw Error(GBCC_ERR_STATE, "gbcc_set_df_inputs: the handle holds integral-direct inputs");
    if (h->S.naux != nq)
      throw Error(GBCC_ERR_STATE, h->S.naux == 0 ? "gbcc_set_df_inputs: the handle holds standard inputs"
                                                 : "gbcc_set_df_inputs: the handle was set up for another naux");
    gbcc::CcsdTensors& S = h->S;
    h->inputs_set = false;
    h->have_solution = false;
    h->seeded = false;
    copy_in(S.eps_o->d, in->eps_o, o, h->stream);
    copy_in(S.eps_v->d, in->eps_v, v, h->stream);
    copy_in(S.Fia->d, in->Fia, o * v, h->stream);
    copy_in(S.Fij->d, in->Fij, o * o, h->stream);
    copy_in(S.Fab->d, in->Fab, v * v, h->stream);
    copy_in(S.Gijab->d, in->Gijab, o * o * v * v, h->stream);
    copy_in(S.Gijkl->d, in->Gijkl, o * o * o * o, h->stream);
    copy_in(S.Giajb->d, in->Giajb, o * v * o * v, h->stream);
    copy_in(S.Gijka->d, in->Gijka, o * o * o * v, h->stream);
    copy_in(S.Xai->d, in->Xai, nq * v * o, h->stream);
    copy_in(S.Xab->d, in->Xab, nq * v * v, h->stream);
    commit_inputs(h);
    return GBCC_OK;
  });
}

gbcc_status gbcc_set_direct_inputs(gbcc_handle* h, const gbcc_direct_inputs* in) {
  return guarded(h, [&]() -> gbcc_status {
    if (!in) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_direct_inputs: NULL inputs");
    const double* ptrs[] = {in->eps_o, in->eps_v, in->Fia, in->Fij, in->Fab, in->Gijab, in->Gijkl,
                            in->Giajb, in->Gijka, in->Giabc, in->Gao, in->Ca, in->Ci};
    for (const double* p : ptrs)
      if (!p) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_direct_inputs: NULL input array");
    const int64_t o = h->cfg.o, v = h->cfg.v, n = in->nao;
    if (n < 1 || n > 1024) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_direct_inputs: nao must be 1..1024");
    validate_eps(in->eps_o, in->eps_v, o, v);
    create_tensors(h, 0, n);
    if (h->S.naux > 0) throw Error(GBCC_ERR_STATE, "gbcc_set_direct_inputs: the handle holds density-fitted inputs");
    if (h->S.nao != n)
      throw Error(GBCC_ERR_STATE, h->S.nao == 0 ? "gbcc_set_direct_inputs: the handle holds standard inputs"
                                                : "gbcc_set_direct_inputs: the handle was set up for another nao");
    gbcc::CcsdTensors& S = h->S;
    h->inputs_set = false;
    h->have_solution = false;
    h->seeded = false;
    copy_in(S.eps_o->d, in->eps_o, o, h->stream);
    copy_in(S.eps_v->d, in->eps_v, v, h->stream);
    copy_in(S.Fia->d, in->Fia, o * v, h->stream);
    copy_in(S.Fij->d, in->Fij, o * o, h->stream);
    copy_in(S.Fab->d, in->Fab, v * v, h->stream);
    copy_in(S.Gijab->d, in->Gijab, o * o * v * v, h->stream);
    copy_in(S.Gijkl->d, in->Gijkl, o * o * o * o, h->stream);
    copy_in(S.Giajb->d, in->Giajb, o * v * o * v, h->stream);
    copy_in(S.Gijka->d, in->Gijka, o * o * o * v, h->stream);
    copy_in(S.Giabc->d, in->Giabc, o * v * v * v, h->stream);
    copy_in(S.Gao->d, in->Gao, n * n * n * n, h->stream);
    copy_in(S.Ca->d, in->Ca, n * v, h->stream);
    copy_in(S.Ci->d, in->Ci, n * o, h->stream);
    commit_inputs(h);
    return GBCC_OK;
  });
}

gbcc_status gbcc_device_inputs(gbcc_handle* h, gbcc_inputs* out) {
  return guarded(h, [&]() -> gbcc_status {
    if (!out) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_device_inputs: NULL output");
    create_tensors(h, 0, 0);
    if (h->S.naux > 0 || h->S.nao > 0)
      throw Error(GBCC_ERR_STATE, "gbcc_device_inputs: the handle holds density-fitted or integral-direct inputs");
    gbcc::CcsdTensors& S = h->S;
    h->eng->acquire(*S.Gabcd);  // given back by the previous commit
    GBCC_CK(cudaStreamSynchronize(h->stream));  // zero-initialisation done
    out->eps_o = S.eps_o->d;
    out->eps_v = S.eps_v->d;
    out->Fia = S.Fia->d;
    out->Fij = S.Fij->d;
    out->Fab = S.Fab->d;
    out->Gijab = S.Gijab->d;
    out->Gijkl = S.Gijkl->d;
    out->Giajb = S.Giajb->d;
    out->Gijka = S.Gijka->d;
    out->Giabc = S.Giabc->d;
    out->Gabcd = S.Gabcd->d;
    h->inputs_set = false;
    h->have_solution = false;
    h->seeded = false;
    return GBCC_OK;
  });
}

gbcc_status gbcc_commit_inputs(gbcc_handle* h) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->S.t1) throw Error(GBCC_ERR_STATE, "gbcc_commit_inputs: call gbcc_device_inputs first");
    GBCC_CK(cudaStreamSynchronize(h->stream));
    validate_eps(h->S.eps_o->d, h->S.eps_v->d, h->cfg.o, h->cfg.v);
    commit_inputs(h);
    return GBCC_OK;
  });
}

gbcc_status gbcc_residual_ex(gbcc_handle* h, int32_t precision, const double* t1_ai,
                             const double* t2_abij, double* r1_ai, double* r2_abij) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "gbcc_residual: inputs not set");
    if (precision != GBCC_PREC_FP64 && precision != GBCC_PREC_MIXED && precision != GBCC_PREC_FP64_TC)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_residual: bad precision");
    if (precision == GBCC_PREC_FP64_TC && !h->eng->emulation())
      throw Error(GBCC_ERR_STATE, "gbcc_residual: the handle has no FP64_TC plan (precision or refine_precision)");
    if (!t1_ai || !t2_abij || !r1_ai || !r2_abij)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_residual: NULL argument");
    h->have_solution = false;
    copy_in(h->S.t1->d, t1_ai, n1_of(h), h->stream);
    copy_in(h->S.t2->d, t2_abij, n2_of(h), h->stream);
    check_pair_symmetric(h);
    run_residual(h, precision);
    copy_out(r1_ai, h->S.r1->d, n1_of(h), h->stream);
    copy_out(r2_abij, h->S.r2->d, n2_of(h), h->stream);
    sync_check(h);
    return GBCC_OK;
  });
}

gbcc_status gbcc_residual(gbcc_handle* h, const double* t1_ai, const double* t2_abij, double* r1_ai,
                          double* r2_abij) {
  if (!h) return GBCC_ERR_INVALID_ARG;
  return gbcc_residual_ex(h, h->cfg.precision, t1_ai, t2_abij, r1_ai, r2_abij);
}

gbcc_status gbcc_energy(gbcc_handle* h, const double* t1_ai, const double* t2_abij, const double* r1_ai,
                        const double* r2_abij, double* energy, double* error) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "gbcc_energy: inputs not set");
    if (!t1_ai || !t2_abij || !r1_ai || !r2_abij)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_energy: NULL argument");
    h->have_solution = false;
    copy_in(h->S.t1->d, t1_ai, n1_of(h), h->stream);
    copy_in(h->S.t2->d, t2_abij, n2_of(h), h->stream);
    copy_in(h->S.r1->d, r1_ai, n1_of(h), h->stream);
    copy_in(h->S.r2->d, r2_abij, n2_of(h), h->stream);
    gbcc::launch_make_tau(h->cfg.o, h->cfg.v, h->S.t1->d, h->S.t2->d, h->S.tau->d, h->stream);
    auto ee = energy_error(h);
    if (energy) *energy = ee.first;
    if (error) *error = ee.second;
    return GBCC_OK;
  });
}

gbcc_status gbcc_solve(gbcc_handle* h, double* t1_ai, double* t2_abij, double* e_corr,
                       gbcc_report* report) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "gbcc_solve: inputs not set");
    const gbcc_config& c = h->cfg;
    gbcc::CcsdTensors& S = h->S;
    const int64_t n1 = n1_of(h), n2 = n2_of(h);
    ensure_diis(h);
    gbcc_report rep{};
    h->have_solution = false;
    bool mixed_phase = c.precision == GBCC_PREC_MIXED;
    const bool used_mixed = mixed_phase;
    int fp64_resid = 0, mixed_resid = 0;
    double t_mixed = 0.0, t_fp64 = 0.0;
    GBCC_CK(cudaMemsetAsync(h->Bmat, 0, c.n_diis * c.n_diis * sizeof(double), h->stream));
    if (h->seeded) {
      // restart: the residual of the seeded amplitudes in the starting precision
      GBCC_CK(cudaMemcpyAsync(S.t1->d, h->seed1, n1 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
      GBCC_CK(cudaMemcpyAsync(S.t2->d, h->seed2, n2 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
      h->seeded = false;
      const int prec = mixed_phase ? GBCC_PREC_MIXED : hi_prec(h);
      GBCC_CK(cudaEventRecord(h->ev0, h->stream));
      run_residual(h, prec);
      GBCC_CK(cudaEventRecord(h->ev1, h->stream));
      sync_check(h);
      float ms = 0.f;
      GBCC_CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
      if (prec == GBCC_PREC_MIXED) {
        ++mixed_resid;
        t_mixed += ms * 1e-3;
      } else {
        ++fp64_resid;
        t_fp64 += ms * 1e-3;
      }
    } else {
      // t = 0, tau = 0, r1 = f_ai, r2 = g_abij   (ccsd.h:331-350)
      GBCC_CK(cudaMemsetAsync(S.t1->d, 0, n1 * sizeof(double), h->stream));
      GBCC_CK(cudaMemsetAsync(S.t2->d, 0, n2 * sizeof(double), h->stream));
      GBCC_CK(cudaMemsetAsync(S.tau->d, 0, n2 * sizeof(double), h->stream));
      GBCC_CK(cudaMemcpyAsync(S.r1->d, S.f_ai->d, n1 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
      GBCC_CK(cudaMemcpyAsync(S.r2->d, S.g_abij->d, n2 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    }
    bool reset_after_update = false;
    double E1 = 0.0, E0 = 0.0, dE = 0.0, error = 1.0;
    double best_error = std::numeric_limits<double>::infinity();
    double best_dE = std::numeric_limits<double>::infinity();
    int stalled = 0;
    int iter = 0;
    bool converged = false;
    int diis_iter = 0, nvec = 0, head = -1;
    std::vector<int> slots;  // age order
    auto wall0 = std::chrono::steady_clock::now();
    const bool graph_solve = c.use_graphs == 2 && !h->profiling && !h->calibrating;
    if (graph_solve) {
      // the whole loop below, decided on the device: one launch, one synchronisation
      if (!h->solve_exec) build_solve_graph(h);
      gbcc::launch_solve_init(h->d_state, mixed_phase ? 1 : 0, h->stream);
      GBCC_CK(cudaGraphLaunch(h->solve_exec, h->stream));
      sync_check(h);
      gbcc::SolveState ss{};
      read_back(h, &ss, h->d_state, sizeof(ss));
      const int ntest = ss.iter + (ss.stop ? 1 : 0);
      std::vector<double> hist(3 * static_cast<size_t>(std::max(ntest, 1)));
      std::vector<unsigned long long> stamps(2 * static_cast<size_t>(std::max(ss.iter, 1)));
      if (ntest > 0)
        read_back(h, hist.data(), h->d_history, 3 * ntest * sizeof(double));
      if (ss.iter > 0)
        read_back(h, stamps.data(), h->d_stamps, 2 * ss.iter * sizeof(unsigned long long));
      if (ss.status) throw Error(GBCC_ERR_NUMERIC, "non-finite energy or residual at iteration " + std::to_string(ss.iter));
      for (int k = 0; k < ss.iter; ++k) {
        const double secs_k = static_cast<double>(stamps[2 * k + 1] - stamps[2 * k]) * 1e-9;
        if (k < ss.mixed_resid)
          t_mixed += secs_k;
        else
          t_fp64 += secs_k;
      }
      mixed_resid += ss.mixed_resid;
      fp64_resid += ss.fp64_resid;
      iter = ss.iter;
      converged = ss.converged != 0;
      E1 = ss.E1;
      dE = ss.dE;
      error = ss.error;
      if (c.verbose)
        for (int k = 1; k < ntest; ++k) print_iter(k, hist[3 * k + 1], hist[3 * k + 2], hist[3 * k], 0.0);
    }
    while (!graph_solve && iter < c.max_iter) {
      auto ee = energy_error(h);
      error = ee.second;
      E0 = E1;
      E1 = ee.first;
      dE = std::fabs(E0 - E1);
      if (!std::isfinite(E1) || !std::isfinite(error))
        throw Error(GBCC_ERR_NUMERIC, "non-finite energy or residual at iteration " + std::to_string(iter));
      const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
      if (c.verbose && iter > 0) print_iter(iter, dE, error, E1, secs);
      bool conv = iter > 0 && error <= c.target_precision && dE <= 0.1 * c.target_precision;
      if (mixed_phase) {
        // The split-precision phase ends once it has converged on its own residual
        // (switch precision, default the target) or once it stops making progress:
        // near its fixed point the split map has a rounding floor below which
        // neither dE nor the error shrinks (DIIS otherwise sets a new minimum of
        // both every iteration or two).  The FP64 iterations then absorb the
        // split error.
        const double sw = c.mixed_switch_precision > 0.0 ? c.mixed_switch_precision : c.target_precision;
        if (iter > 0) {
          bool progress = false;
          if (error < 0.5 * best_error) {
            best_error = error;
            progress = true;
          }
          if (dE < 0.5 * best_dE) {
            best_dE = dE;
            progress = true;
          }
          stalled = progress ? 0 : stalled + 1;
          if ((error <= sw && dE <= 0.1 * sw) || stalled >= 4) {
            mixed_phase = false;
            reset_after_update = c.refine_reset_diis != 0;
          }
        }
        conv = false;
      } else if (used_mixed && fp64_resid < c.refine_iters) {
        conv = false;
      }
      if (iter != 0 && conv) {
        converged = true;
        break;
      }
      // Jacobi update + DIIS (cc/solvers.h:112-121; lcao/cc/solvers.h:1152-1158)
      ++diis_iter;
      head = (head + 1) % c.n_diis;
      if (nvec == c.n_diis) slots.erase(slots.begin());
      else ++nvec;
      slots.push_back(head);
      gbcc::DiisArgs d{};
      d.o = c.o;
      d.v = c.v;
      d.eps_o = S.eps_o->d;
      d.eps_v = S.eps_v->d;
      d.dinv1 = S.Dinv1->d;
      d.dinv2 = S.Dinv2->d;
      d.t1 = S.t1->d;
      d.t2 = S.t2->d;
      d.r1 = S.r1->d;
      d.r2 = S.r2->d;
      d.x1 = h->x1;
      d.x2 = h->x2;
      d.e1 = h->e1;
      d.e2 = h->e2;
      d.ndiis = c.n_diis;
      d.slot = head;
      d.nvec = nvec;
      for (int q = 0; q < nvec; ++q) d.slots[q] = slots[q];
      d.partial = h->d_partial;
      d.Bmat = h->Bmat;
      d.coef = h->coef;
      d.damping = c.diis_damp;
      bool extrap = diis_iter >= c.diis_start;
      if (c.diis_ngroup > 1 && (diis_iter - c.diis_start) % c.diis_ngroup >= c.diis_group_nstart)
        extrap = false;
      d.extrapolate = extrap ? 1 : 0;
      d.nskip_out = h->d_nskip;
      gbcc::launch_diis_step(d, h->stream);
      gbcc::launch_diis_extrapolate(c.o, c.v, h->x1, h->x2, h->coef, c.n_diis, slots.data(), nvec,
                                    S.t1->d, S.t2->d, S.tau->d, h->stream);
      if (reset_after_update) {
        // a new subspace for the FP64 refinement: only FP64 residuals from here on
        reset_after_update = false;
        diis_iter = 0;
        nvec = 0;
        head = -1;
        slots.clear();
        GBCC_CK(cudaMemsetAsync(h->Bmat, 0, c.n_diis * c.n_diis * sizeof(double), h->stream));
      }
      // residual of the new amplitudes
      const int prec = mixed_phase ? GBCC_PREC_MIXED : hi_prec(h);
      GBCC_CK(cudaEventRecord(h->ev0, h->stream));
      h->last_launches = enqueue_residual_program(h, prec);
      GBCC_CK(cudaEventRecord(h->ev1, h->stream));
      sync_check(h);
      float ms = 0.f;
      GBCC_CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
      if (prec == GBCC_PREC_MIXED) {
        ++mixed_resid;
        t_mixed += ms * 1e-3;
      } else {
        ++fp64_resid;
        t_fp64 += ms * 1e-3;
      }
      ++iter;
    }
    if (!converged && c.verbose) std::printf("\n Warning!! Exceed Max Iteration! \n");
    if (t1_ai) copy_out(t1_ai, S.t1->d, n1, h->stream);
    if (t2_abij) copy_out(t2_abij, S.t2->d, n2, h->stream);
    sync_check(h);
    if (e_corr) *e_corr = E1;
    h->have_solution = true;
    h->last_e = E1;
    rep.iters = iter;
    rep.converged = converged ? 1 : 0;
    rep.mixed_iters = mixed_resid;
    rep.fp64_iters = fp64_resid;
    rep.e_corr = E1;
    rep.last_dE = dE;
    rep.last_error = error;
    rep.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    rep.seconds_residual_mixed = mixed_resid ? t_mixed / mixed_resid : 0.0;
    rep.seconds_residual_fp64 = fp64_resid ? t_fp64 / fp64_resid : 0.0;
    if (report) *report = rep;
    if (c.verbose) std::printf("CCSD Energy  %.15f\n", E1);
    return converged ? GBCC_OK : GBCC_ERR_NOT_CONVERGED;
  });
}

gbcc_status gbcc_triples(gbcc_handle* h, int32_t precision, const double* t1_ai, const double* t2_abij,
                         double* e_t) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "gbcc_triples: inputs not set");
    if (precision != GBCC_PREC_FP64 && precision != GBCC_PREC_MIXED && precision != GBCC_PREC_FP64_TC)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_triples: bad precision");
    if (!e_t) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_triples: NULL e_t");
    if ((t1_ai == nullptr) != (t2_abij == nullptr))
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_triples: give both amplitudes or neither");
    gbcc::CcsdTensors& S = h->S;
    if (t1_ai) {
      h->have_solution = false;
      copy_in(S.t1->d, t1_ai, n1_of(h), h->stream);
      copy_in(S.t2->d, t2_abij, n2_of(h), h->stream);
      check_pair_symmetric(h);
    } else if (!h->have_solution) {
      throw Error(GBCC_ERR_STATE, "gbcc_triples: no amplitudes given and no solve to take them from");
    }
    gbcc::TriplesInputs in;
    in.o = h->cfg.o;
    in.v = h->cfg.v;
    in.t1 = S.t1->d;
    in.t2 = S.t2->d;
    in.Gijab = S.Gijab->d;
    in.Gijka = S.Gijka->d;
    in.Giabc = S.Giabc->d;
    in.eps_o = S.eps_o->d;
    in.eps_v = S.eps_v->d;
    *e_t = gbcc::triples_energy(in, precision, h->stream, h->d_err);
    sync_check(h);
    return GBCC_OK;
  });
}

gbcc_status gbcc_solve_batch(gbcc_handle* const* handles, int32_t count, double* e_corr, gbcc_report* reports,
                             gbcc_status* statuses) {
  if (!handles || count < 0) return GBCC_ERR_INVALID_ARG;
  for (int32_t k = 0; k < count; ++k)
    if (!handles[k]) return GBCC_ERR_INVALID_ARG;
  for (int32_t k = 0; k < count; ++k)
    for (int32_t q = 0; q < k; ++q)
      if (handles[q] == handles[k]) {
        handles[k]->last_error = "gbcc_solve_batch: a handle appears twice";
        return GBCC_ERR_INVALID_ARG;
      }
  std::vector<gbcc_status> st(count, GBCC_OK);
  std::vector<gbcc_report> rep(count);
  std::vector<double> e(count, 0.0);
  std::vector<std::thread> threads;
  threads.reserve(count);
  for (int32_t k = 0; k < count; ++k)
    threads.emplace_back([&, k] { st[k] = gbcc_solve(handles[k], nullptr, nullptr, &e[k], &rep[k]); });
  for (auto& t : threads) t.join();
  gbcc_status out = GBCC_OK;
  for (int32_t k = 0; k < count; ++k) {
    if (e_corr) e_corr[k] = e[k];
    if (reports) reports[k] = rep[k];
    if (statuses) statuses[k] = st[k];
    if (st[k] != GBCC_OK && st[k] != GBCC_ERR_NOT_CONVERGED && (out == GBCC_OK || out == GBCC_ERR_NOT_CONVERGED))
      out = st[k];
    else if (st[k] == GBCC_ERR_NOT_CONVERGED && out == GBCC_OK)
      out = GBCC_ERR_NOT_CONVERGED;
  }
  return out;
}

gbcc_status gbcc_destroy(gbcc_handle* h) {
  if (!h) return GBCC_OK;
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  h->eng.reset();
  h->aux.reset();
  for (void* p : {(void*)h->x1, (void*)h->x2, (void*)h->e1, (void*)h->e2, (void*)h->Bmat, (void*)h->coef,
                  (void*)h->d_nskip, (void*)h->d_err, (void*)h->d_partial, (void*)h->d_out,
                  (void*)h->seed1, (void*)h->seed2, (void*)h->d_state, (void*)h->d_history, (void*)h->d_stamps})
    gbcc::dev_free(p);
  if (h->h_out) cudaFreeHost(h->h_out);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (cudaEvent_t e : h->slots)
    if (e) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return GBCC_OK;
}

gbcc_status gbcc_set_amplitudes(gbcc_handle* h, const double* t1_ai, const double* t2_abij) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "gbcc_set_amplitudes: inputs not set");
    if (!t1_ai || !t2_abij) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_set_amplitudes: NULL amplitudes");
    const int64_t n1 = n1_of(h), n2 = n2_of(h);
    if (!h->seed1) h->seed1 = static_cast<double*>(gbcc::dev_alloc(n1 * sizeof(double)));
    if (!h->seed2) h->seed2 = static_cast<double*>(gbcc::dev_alloc(n2 * sizeof(double)));
    copy_in(h->seed1, t1_ai, n1, h->stream);
    copy_in(h->seed2, t2_abij, n2, h->stream);
    // the pair-symmetry check reads S.t2: stage the seed there
    GBCC_CK(cudaMemcpyAsync(h->S.t2->d, h->seed2, n2 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    h->have_solution = false;
    check_pair_symmetric(h);
    h->seeded = true;
    return GBCC_OK;
  });
}

namespace {
constexpr char kAmpMagic[8] = {'G', 'B', 'C', 'C', 'A', 'M', 'P', '1'};
struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};
}  // namespace

gbcc_status gbcc_save_amplitudes(gbcc_handle* h, const char* path) {
  return guarded(h, [&]() -> gbcc_status {
    if (!path) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_save_amplitudes: NULL path");
    if (!h->have_solution) throw Error(GBCC_ERR_STATE, "gbcc_save_amplitudes: no solve has completed");
    const int64_t n1 = n1_of(h), n2 = n2_of(h);
    std::vector<double> t1(n1), t2(n2);
    GBCC_CK(cudaMemcpyAsync(t1.data(), h->S.t1->d, n1 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    GBCC_CK(cudaMemcpyAsync(t2.data(), h->S.t2->d, n2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    GBCC_CK(cudaStreamSynchronize(h->stream));
    FileCloser fc{std::fopen(path, "wb")};
    if (!fc.f) throw Error(GBCC_ERR_INVALID_ARG, std::string("gbcc_save_amplitudes: cannot open ") + path);
    const int64_t dims[2] = {h->cfg.o, h->cfg.v};
    const bool ok = std::fwrite(kAmpMagic, 1, 8, fc.f) == 8 && std::fwrite(dims, sizeof(int64_t), 2, fc.f) == 2 &&
                    std::fwrite(&h->last_e, sizeof(double), 1, fc.f) == 1 &&
                    std::fwrite(t1.data(), sizeof(double), n1, fc.f) == static_cast<size_t>(n1) &&
                    std::fwrite(t2.data(), sizeof(double), n2, fc.f) == static_cast<size_t>(n2);
    if (!ok || std::fflush(fc.f) != 0) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_save_amplitudes: write failed");
    return GBCC_OK;
  });
}

gbcc_status gbcc_load_amplitudes(gbcc_handle* h, const char* path, double* e_corr) {
  return guarded(h, [&]() -> gbcc_status {
    if (!path) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_load_amplitudes: NULL path");
    FileCloser fc{std::fopen(path, "rb")};
    if (!fc.f) throw Error(GBCC_ERR_INVALID_ARG, std::string("gbcc_load_amplitudes: cannot open ") + path);
    char magic[8];
    int64_t dims[2];
    double e = 0.0;
    if (std::fread(magic, 1, 8, fc.f) != 8 || std::memcmp(magic, kAmpMagic, 8) != 0 ||
        std::fread(dims, sizeof(int64_t), 2, fc.f) != 2 || std::fread(&e, sizeof(double), 1, fc.f) != 1)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_load_amplitudes: not an amplitude checkpoint");
    if (dims[0] != h->cfg.o || dims[1] != h->cfg.v)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_load_amplitudes: checkpoint has o = " + std::to_string(dims[0]) +
                                            ", v = " + std::to_string(dims[1]));
    const int64_t n1 = n1_of(h), n2 = n2_of(h);
    std::vector<double> t1(n1), t2(n2);
    if (std::fread(t1.data(), sizeof(double), n1, fc.f) != static_cast<size_t>(n1) ||
        std::fread(t2.data(), sizeof(double), n2, fc.f) != static_cast<size_t>(n2))
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_load_amplitudes: truncated checkpoint");
    for (double x : t1)
      if (!std::isfinite(x)) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_load_amplitudes: non-finite amplitude");
    std::fclose(fc.f);
    fc.f = nullptr;
    const gbcc_status st = gbcc_set_amplitudes(h, t1.data(), t2.data());
    if (st != GBCC_OK) throw Error(st, h->last_error);
    if (e_corr) *e_corr = e;
    return GBCC_OK;
  });
}

gbcc_status gbcc_autotune_save(const char* path) {
  if (!path) {
    gbcc_set_thread_error("gbcc_autotune_save: NULL path");
    return GBCC_ERR_INVALID_ARG;
  }
  if (!gbcc::tune_save(path)) {
    gbcc_set_thread_error(std::string("gbcc_autotune_save: cannot write ") + path);
    return GBCC_ERR_INVALID_ARG;
  }
  return GBCC_OK;
}

gbcc_status gbcc_autotune_load(const char* path) {
  if (!path || !gbcc::tune_load(path)) {
    gbcc_set_thread_error(std::string("gbcc_autotune_load: cannot read an autotune table from ") +
                          (path ? path : "NULL"));
    return GBCC_ERR_INVALID_ARG;
  }
  return GBCC_OK;
}

gbcc_status gbcc_autotune_clear(void) {
  gbcc::tune_clear();
  return GBCC_OK;
}

gbcc_status gbcc_calibrate_slices(gbcc_handle* h, const double* t1_ai, const double* t2_abij) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "gbcc_calibrate_slices: inputs not set");
    if (h->cfg.precision != GBCC_PREC_MIXED) throw Error(GBCC_ERR_STATE, "gbcc_calibrate_slices: not a mixed-precision handle");
    if (!t1_ai || !t2_abij) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_calibrate_slices: NULL amplitudes");
    h->inputs_set = false;
    h->have_solution = false;
    h->seeded = false;
    calibrate_slices(h, t1_ai, t2_abij);
    h->inputs_set = true;
    return GBCC_OK;
  });
}

gbcc_status gbcc_slice_policy(gbcc_handle* h, int32_t slices[3], double rel_change[3]) {
  if (!h || !slices) return GBCC_ERR_INVALID_ARG;
  if (!h->inputs_set) return fail(h, GBCC_ERR_STATE, "gbcc_slice_policy: inputs not set");
  for (int k = 0; k < 3; ++k) {
    slices[k] = h->slices_used[k];
    if (rel_change) rel_change[k] = h->slice_err[k];
  }
  return GBCC_OK;
}

const char* gbcc_last_error(const gbcc_handle* h) {
  if (!h) return g_create_error.c_str();
  return h->last_error.c_str();
}


int gbcc_testing_profile_residual(gbcc_handle* h, int precision, int max_sites, double* ms, double* flops,
                                  int* pairs, int* cls, int* nsites) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "profile: inputs not set");
    if (precision != GBCC_PREC_FP64 && precision != GBCC_PREC_MIXED && precision != GBCC_PREC_FP64_TC)
      throw Error(GBCC_ERR_INVALID_ARG, "profile: bad precision");
    if (precision == GBCC_PREC_FP64_TC && !h->eng->emulation())
      throw Error(GBCC_ERR_STATE, "profile: the handle has no FP64_TC plan");
    h->eng->set_profile(true);
    h->profiling = true;
    try {
      run_residual(h, precision);
      sync_check(h);
    } catch (...) {
      h->eng->set_profile(false);
      h->profiling = false;
      throw;
    }
    h->eng->set_profile(false);
    h->profiling = false;
    const auto st = h->eng->site_stats(precision);
    h->prof_gemm_ms.clear();
    h->prof_dims.clear();
    h->prof_tiles.clear();
    for (const auto& x : st) {
      h->prof_gemm_ms.push_back(x.gemm_ms);
      h->prof_dims.push_back({x.M, x.N, x.K});
      h->prof_tiles.push_back({x.bn, x.ksplit, x.sps, x.group});
    }
    if (nsites) *nsites = static_cast<int>(st.size());
    for (int i = 0; i < max_sites && i < static_cast<int>(st.size()); ++i) {
      if (ms) ms[i] = st[i].ms;
      if (flops) flops[i] = st[i].flops;
      if (pairs) pairs[i] = st[i].pairs;
      if (cls) cls[i] = st[i].cls;
    }
    return GBCC_OK;
  });
}

int gbcc_testing_profile_gemm_ms(gbcc_handle* h, int max_sites, double* ms) {
  if (!h || !ms) return GBCC_ERR_INVALID_ARG;
  for (int i = 0; i < max_sites && i < static_cast<int>(h->prof_gemm_ms.size()); ++i) ms[i] = h->prof_gemm_ms[i];
  return GBCC_OK;
}

int gbcc_testing_profile_tiles(gbcc_handle* h, int max_sites, int32_t* tiles) {
  if (!h || !tiles) return GBCC_ERR_INVALID_ARG;
  for (int i = 0; i < max_sites && i < static_cast<int>(h->prof_tiles.size()); ++i)
    for (int k = 0; k < 4; ++k) tiles[4 * i + k] = h->prof_tiles[i][k];
  return GBCC_OK;
}

int gbcc_testing_profile_dims(gbcc_handle* h, int max_sites, int64_t* mnk) {
  if (!h || !mnk) return GBCC_ERR_INVALID_ARG;
  for (int i = 0; i < max_sites && i < static_cast<int>(h->prof_dims.size()); ++i)
    for (int k = 0; k < 3; ++k) mnk[3 * i + k] = h->prof_dims[i][k];
  return GBCC_OK;
}

int gbcc_testing_record(gbcc_handle* h, int slot) {
  if (!h || slot < 0 || slot >= 8) return GBCC_ERR_INVALID_ARG;
  return guarded(h, [&]() -> gbcc_status {
    if (!h->slots[slot]) GBCC_CK(cudaEventCreate(&h->slots[slot]));
    GBCC_CK(cudaEventRecord(h->slots[slot], h->stream));
    return GBCC_OK;
  });
}

int gbcc_testing_elapsed(gbcc_handle* h, int slot0, int slot1, float* ms) {
  if (!h || !ms || slot0 < 0 || slot0 >= 8 || slot1 < 0 || slot1 >= 8) return GBCC_ERR_INVALID_ARG;
  return guarded(h, [&]() -> gbcc_status {
    if (!h->slots[slot0] || !h->slots[slot1]) throw Error(GBCC_ERR_STATE, "event slot not recorded");
    GBCC_CK(cudaEventSynchronize(h->slots[slot1]));
    GBCC_CK(cudaEventElapsedTime(ms, h->slots[slot0], h->slots[slot1]));
    return GBCC_OK;
  });
}

int gbcc_testing_tc_launches_total(gbcc_handle* h, int64_t* launches) {
  if (!h || !launches || !h->eng) return GBCC_ERR_INVALID_ARG;
  *launches = h->eng->gemm_tc_launches_total();
  return GBCC_OK;
}

int gbcc_testing_last_launches(gbcc_handle* h, int* launches) {
  if (!h || !launches) return GBCC_ERR_INVALID_ARG;
  *launches = h->last_launches;
  return GBCC_OK;
}

}  // extern "C"
