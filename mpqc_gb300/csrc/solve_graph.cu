// Device side of the whole-solve CUDA graph: the per-iteration decision of
// CCSD::compute_ccsd (src/mpqc/chemistry/qc/lcao/cc/ccsd.h:367-468) and
// DIISSolver (src/mpqc/chemistry/qc/cc/solvers.h:112-121, 141-152) on one
// thread, driving the graph's conditional nodes:
//
//   while (loop) {                      WHILE node, condition `loop`
//     energy terms -> decide            E, error, convergence test, phase switch,
//                                       DIIS slots; sets the conditions below
//     if (update)  Jacobi + DIIS        IF node
//     if (fp64)    residual (FP64)        IF node (child graph)
//     if (mixed)   residual (split BF16)  IF node (child graph)
//   }
//
// It makes the same decisions, in the same order, as the host loop of
// gbcc_solve (api.cpp), so both give identical iterations and energies.
#include "kernels.h"

namespace gbcc {
namespace {

__global__ void solve_init_kernel(SolveState* s, int mixed) {
  SolveState z{};
  z.mixed_phase = mixed;
  z.used_mixed = mixed;
  z.best_error = __longlong_as_double(0x7ff0000000000000LL);  // +inf
  z.best_dE = z.best_error;
  z.head = -1;
  *s = z;
}

__global__ void solve_decide_kernel(SolveParams p) {
  SolveState& s = *p.state;
  if (s.pending_reset) {
    // a new DIIS subspace for the FP64 refinement (requested at the previous update)
    s.pending_reset = 0;
    s.diis_iter = 0;
    s.diis.nvec = 0;
    s.head = -1;
    for (int k = 0; k < p.n_diis * p.n_diis; ++k) p.Bmat[k] = 0.0;
  }
  const double E = 2.0 * p.sums[2] + p.sums[3];
  const double err = sqrt(p.sums[0] + p.sums[1]) / static_cast<double>(p.n1 + p.n2);
  s.E0 = s.E1;
  s.E1 = E;
  s.dE = fabs(s.E0 - s.E1);
  s.error = err;
  p.history[3 * s.iter + 0] = E;
  p.history[3 * s.iter + 1] = s.dE;
  p.history[3 * s.iter + 2] = err;
  bool stop = false, reset_after = false;
  if (!isfinite(E) || !isfinite(err)) {
    s.status = 1;
    stop = true;
  } else {
    bool conv = s.iter > 0 && err <= p.target && s.dE <= 0.1 * p.target;
    if (s.mixed_phase) {
      const double sw = p.switch_precision > 0.0 ? p.switch_precision : p.target;
      if (s.iter > 0) {
        bool progress = false;
        if (err < 0.5 * s.best_error) {
          s.best_error = err;
          progress = true;
        }
        if (s.dE < 0.5 * s.best_dE) {
          s.best_dE = s.dE;
          progress = true;
        }
        s.stalled = progress ? 0 : s.stalled + 1;
        if ((err <= sw && s.dE <= 0.1 * sw) || s.stalled >= 4) {
          s.mixed_phase = 0;
          reset_after = p.reset_diis != 0;
        }
      }
      conv = false;
    } else if (s.used_mixed && s.fp64_resid < p.refine_iters) {
      conv = false;
    }
    if (s.iter != 0 && conv) {
      s.converged = 1;
      stop = true;
    }
  }
  if (stop) {
    s.stop = 1;
    cudaGraphSetConditional(p.cond_update, 0);
    cudaGraphSetConditional(p.cond_mixed, 0);
    cudaGraphSetConditional(p.cond_fp64, 0);
    cudaGraphSetConditional(p.cond_loop, 0);
    return;
  }
  // Jacobi update + DIIS slot of this iteration
  ++s.diis_iter;
  s.head = (s.head + 1) % p.n_diis;
  if (s.diis.nvec == p.n_diis) {
    for (int q = 0; q + 1 < s.diis.nvec; ++q) s.diis.slots[q] = s.diis.slots[q + 1];
  } else {
    ++s.diis.nvec;
  }
  s.diis.slots[s.diis.nvec - 1] = s.head;
  s.diis.slot = s.head;
  bool extrap = s.diis_iter >= p.diis_start;
  if (p.diis_ngroup > 1 && (s.diis_iter - p.diis_start) % p.diis_ngroup >= p.diis_group_nstart) extrap = false;
  s.diis.extrapolate = extrap ? 1 : 0;
  if (reset_after) s.pending_reset = 1;
  const int mixed = s.mixed_phase;
  if (mixed)
    ++s.mixed_resid;
  else
    ++s.fp64_resid;
  ++s.iter;
  cudaGraphSetConditional(p.cond_update, 1);
  cudaGraphSetConditional(p.cond_mixed, mixed ? 1u : 0u);
  cudaGraphSetConditional(p.cond_fp64, mixed ? 0u : 1u);
  cudaGraphSetConditional(p.cond_loop, s.iter < p.max_iter ? 1u : 0u);
}

// timestamps around the residual of the current iteration (iteration iter-1)
__global__ void stamp_kernel(unsigned long long* base, const SolveState* s, int which) {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  base[2 * (s->iter - 1) + which] = t;
}

}  // namespace

void launch_solve_init(SolveState* s, int mixed, cudaStream_t st) { solve_init_kernel<<<1, 1, 0, st>>>(s, mixed); }

void launch_solve_decide(const SolveParams& p, cudaStream_t st) { solve_decide_kernel<<<1, 1, 0, st>>>(p); }

void launch_stamp(unsigned long long* base, const SolveState* s, int which, cudaStream_t st) {
  stamp_kernel<<<1, 1, 0, st>>>(base, s, which);
}

cudaError_t add_stamp_node(cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps, unsigned long long* base,
                           const SolveState* s, int which, cudaGraphNode_t* out) {
  void* args[] = {&base, &s, &which};
  cudaKernelNodeParams kp{};
  kp.func = reinterpret_cast<void*>(stamp_kernel);
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(1);
  kp.kernelParams = args;
  return cudaGraphAddKernelNode(out, g, deps, ndeps, &kp);
}

}  // namespace gbcc
