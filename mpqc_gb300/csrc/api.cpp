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
#include <utility>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbcc.h"
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
  bool prepacked = false;
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

void copy_in(double* dst, const double* src, int64_t n, cudaStream_t st) {
  GBCC_CK(cudaMemcpyAsync(dst, src, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDefault, st));
}

void copy_out(double* dst, const double* src, int64_t n, cudaStream_t st) {
  GBCC_CK(cudaMemcpyAsync(dst, src, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDefault, st));
}

// Check the device error word and any pending CUDA error after a sync.
void sync_check(gbcc_handle* h) {
  GBCC_CK(cudaStreamSynchronize(h->stream));
  GBCC_CK(cudaGetLastError());
  int err = 0;
  GBCC_CK(cudaMemcpy(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err != gbcc::kDevOk) {
    GBCC_CK(cudaMemset(h->d_err, 0, sizeof(int)));
    throw Error(GBCC_ERR_TIMEOUT, "a bounded device-side wait gave up (tensor-core pipeline)");
  }
}

bool check_config(const gbcc_config* c, std::string& why) {
  if (c->o < 1 || c->v < 1) { why = "o and v must be >= 1"; return false; }
  if (c->o > 4096 || c->v > 8192) { why = "o or v out of range"; return false; }
  if (c->precision != GBCC_PREC_FP64 && c->precision != GBCC_PREC_MIXED) { why = "bad precision"; return false; }
  for (int s : {c->slices_ladder, c->slices_ring, c->slices_other})
    if (s < 1 || s > 3) { why = "slices must be 1..3"; return false; }
  if (c->n_diis < 1 || c->n_diis > 16) { why = "n_diis must be 1..16"; return false; }
  if (c->diis_ngroup < 1 || c->diis_start < 0 || c->diis_group_nstart < 0) { why = "bad DIIS parameters"; return false; }
  if (!(c->diis_damp >= 0.0)) { why = "diis_damp must be >= 0"; return false; }
  if (c->max_iter < 1) { why = "max_iter must be >= 1"; return false; }
  if (!(c->target_precision > 0.0)) { why = "target_precision must be > 0"; return false; }
  if (c->refine_iters < 0) { why = "refine_iters must be >= 0"; return false; }
  return true;
}

void run_residual(gbcc_handle* h, int precision) {
  if (precision == GBCC_PREC_MIXED && !h->prepacked) {
    h->eng->finalize(true);
    h->prepacked = true;
  }
  gbcc::launch_make_tau(h->cfg.o, h->cfg.v, h->S.t1->d, h->S.t2->d, h->S.tau->d, h->stream);
  h->eng->begin(gbcc::Mode::kExec, precision);
  gbcc::residual_program(*h->eng, h->S);
  h->eng->end();
  h->last_launches = 1 + h->eng->kernel_launches();
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

// Derived constants, the residual plan for both precisions and (mixed
// handles) the split copies of the constant operands.
void commit_inputs(gbcc_handle* h) {
  gbcc::CcsdTensors& S = h->S;
  h->aux->reset_plans();
  h->aux->begin(gbcc::Mode::kPlan, GBCC_PREC_FP64);
  gbcc::setup_program(*h->aux, S);
  h->aux->end();
  h->aux->finalize(false);
  h->aux->begin(gbcc::Mode::kExec, GBCC_PREC_FP64);
  gbcc::setup_program(*h->aux, S);
  h->aux->end();
  h->eng->reset_plans();
  h->prepacked = false;
  h->eng->set_frozen({S.t1, S.t2, S.tau});
  h->eng->begin(gbcc::Mode::kPlan, GBCC_PREC_FP64);
  gbcc::residual_program(*h->eng, S);
  h->eng->end();
  const bool mixed = h->cfg.precision == GBCC_PREC_MIXED;
  h->eng->finalize(mixed);
  h->prepacked = mixed;
  sync_check(h);
  h->inputs_set = true;
}

}  // namespace

// Thread-local message read by gbcc_last_error(NULL) (handle-free entry points).
void gbcc_set_thread_error(const std::string& msg) { g_create_error = msg; }

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
  c->slices_ladder = 3;
  c->slices_ring = 3;
  c->slices_other = 3;
  c->refine_iters = 2;
  c->mixed_switch_precision = 1e-7;
  c->max_iter = 30;
  c->target_precision = 1e-9;
  c->diis_start = 1;
  c->n_diis = 8;
  c->diis_damp = 0.0;
  c->diis_ngroup = 1;
  c->diis_group_nstart = 1;
  c->verbose = 0;
  c->device = 0;
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
    if (!h->S.t1) h->S.create(*h->eng, o, v);
    gbcc::CcsdTensors& S = h->S;
    h->inputs_set = false;
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
    copy_in(S.Gabcd->d, in->Gabcd, v * v * v * v, h->stream);
    commit_inputs(h);
    return GBCC_OK;
  });
}

gbcc_status gbcc_device_inputs(gbcc_handle* h, gbcc_inputs* out) {
  return guarded(h, [&]() -> gbcc_status {
    if (!out) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_device_inputs: NULL output");
    if (!h->S.t1) h->S.create(*h->eng, h->cfg.o, h->cfg.v);
    GBCC_CK(cudaStreamSynchronize(h->stream));  // zero-initialisation done
    const gbcc::CcsdTensors& S = h->S;
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
    if (precision != GBCC_PREC_FP64 && precision != GBCC_PREC_MIXED)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_residual: bad precision");
    if (!t1_ai || !t2_abij || !r1_ai || !r2_abij)
      throw Error(GBCC_ERR_INVALID_ARG, "gbcc_residual: NULL argument");
    copy_in(h->S.t1->d, t1_ai, n1_of(h), h->stream);
    copy_in(h->S.t2->d, t2_abij, n2_of(h), h->stream);
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
    // t = 0, tau = 0, r1 = f_ai, r2 = g_abij   (ccsd.h:331-350)
    GBCC_CK(cudaMemsetAsync(S.t1->d, 0, n1 * sizeof(double), h->stream));
    GBCC_CK(cudaMemsetAsync(S.t2->d, 0, n2 * sizeof(double), h->stream));
    GBCC_CK(cudaMemsetAsync(S.tau->d, 0, n2 * sizeof(double), h->stream));
    GBCC_CK(cudaMemcpyAsync(S.r1->d, S.f_ai->d, n1 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    GBCC_CK(cudaMemcpyAsync(S.r2->d, S.g_abij->d, n2 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    GBCC_CK(cudaMemsetAsync(h->Bmat, 0, c.n_diis * c.n_diis * sizeof(double), h->stream));
    bool mixed_phase = c.precision == GBCC_PREC_MIXED;
    const bool used_mixed = mixed_phase;
    int fp64_resid = 0, mixed_resid = 0;
    double t_mixed = 0.0, t_fp64 = 0.0;
    double E1 = 0.0, E0 = 0.0, dE = 0.0, error = 1.0;
    int iter = 0;
    bool converged = false;
    int diis_iter = 0, nvec = 0, head = -1;
    std::vector<int> slots;  // age order
    auto wall0 = std::chrono::steady_clock::now();
    while (iter < c.max_iter) {
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
        if (iter > 0 && error <= c.mixed_switch_precision && dE <= 0.1 * c.mixed_switch_precision)
          mixed_phase = false;
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
      // residual of the new amplitudes
      const int prec = mixed_phase ? GBCC_PREC_MIXED : GBCC_PREC_FP64;
      GBCC_CK(cudaEventRecord(h->ev0, h->stream));
      if (prec == GBCC_PREC_MIXED && !h->prepacked) {
        h->eng->finalize(true);
        h->prepacked = true;
      }
      h->eng->begin(gbcc::Mode::kExec, prec);
      gbcc::residual_program(*h->eng, S);
      h->eng->end();
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

gbcc_status gbcc_destroy(gbcc_handle* h) {
  if (!h) return GBCC_OK;
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->eng.reset();
  h->aux.reset();
  for (void* p : {(void*)h->x1, (void*)h->x2, (void*)h->e1, (void*)h->e2, (void*)h->Bmat, (void*)h->coef,
                  (void*)h->d_nskip, (void*)h->d_err, (void*)h->d_partial, (void*)h->d_out})
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

const char* gbcc_last_error(const gbcc_handle* h) {
  if (!h) return g_create_error.c_str();
  return h->last_error.c_str();
}


int gbcc_testing_profile_residual(gbcc_handle* h, int precision, int max_sites, double* ms, double* flops,
                                  int* pairs, int* cls, int* nsites) {
  return guarded(h, [&]() -> gbcc_status {
    if (!h->inputs_set) throw Error(GBCC_ERR_STATE, "profile: inputs not set");
    if (precision != GBCC_PREC_FP64 && precision != GBCC_PREC_MIXED)
      throw Error(GBCC_ERR_INVALID_ARG, "profile: bad precision");
    h->eng->set_profile(true);
    try {
      run_residual(h, precision);
      sync_check(h);
    } catch (...) {
      h->eng->set_profile(false);
      throw;
    }
    h->eng->set_profile(false);
    const auto st = h->eng->site_stats(precision);
    h->prof_gemm_ms.clear();
    h->prof_dims.clear();
    for (const auto& x : st) {
      h->prof_gemm_ms.push_back(x.gemm_ms);
      h->prof_dims.push_back({x.M, x.N, x.K});
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

int gbcc_testing_last_launches(gbcc_handle* h, int* launches) {
  if (!h || !launches) return GBCC_ERR_INVALID_ARG;
  *launches = h->last_launches;
  return GBCC_OK;
}

}  // extern "C"
