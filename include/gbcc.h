/*
 * gbcc.h -- C ABI of the GB300-native closed-shell CCSD amplitude solver.
 *
 * The library replaces the residual engine and the Jacobi/DIIS iteration of
 * MPQC's closed-shell CCSD (paths relative to the MPQC source tree):
 *
 *   gbcc_create      <- CCSD(const KeyVal&)            src/mpqc/chemistry/qc/lcao/cc/ccsd.h:70-115
 *                       DIISSolver(const KeyVal&)      src/mpqc/chemistry/qc/cc/solvers.h:93-95
 *   gbcc_set_inputs  <- cc::Integrals<Array> members   src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:24-56
 *                       filled in CCSD::compute_ccsd   src/mpqc/chemistry/qc/lcao/cc/ccsd.h:281-296
 *                       and the orbital energies of JacobiDIISSolver
 *                                                      src/mpqc/chemistry/qc/lcao/cc/solvers.h:1128-1136
 *   gbcc_residual    <- compute_cs_ccsd_r1 + compute_cs_ccsd_r2 (standard method)
 *                                                      src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:70-124, 198-293
 *   gbcc_energy      <- the residual-augmented energy  src/mpqc/chemistry/qc/lcao/cc/ccsd.h:377-379
 *                       and Solver::error              src/mpqc/chemistry/qc/cc/solvers.h:60-63
 *   gbcc_solve       <- CCSD::compute_ccsd loop        src/mpqc/chemistry/qc/lcao/cc/ccsd.h:268-477
 *   gbcc_destroy     <- ~CCSD / solver_.reset()        src/mpqc/chemistry/qc/lcao/cc/ccsd.h:246
 *
 * Conventions
 *   - All arrays are dense FP64, row-major, in the index order of the MPQC
 *     annotation: Fia[i][a], Fij[i][j], Fab[a][b], Gijab[i][j][a][b] = <ij|ab>,
 *     Gijkl[i][j][k][l], Giajb[i][a][j][b], Gijka[i][j][k][a],
 *     Giabc[i][a][b][c], Gabcd[a][b][c][d], t1[a][i], t2[a][b][i][j].
 *     o counts the active (correlated) occupied orbitals, v the virtuals.
 *   - Every pointer argument may point to host memory or to device memory of
 *     the handle's GPU; the library detects which.
 *   - The caller owns every array.  gbcc_set_inputs copies the integrals into
 *     handle-owned device memory; no pointer is retained after a call returns.
 *   - One handle per host thread; a handle is not internally locked.
 *   - Every call returns a gbcc_status; no C++ exception crosses the ABI.
 *     gbcc_last_error() gives the message of the last failing call.
 */
#ifndef GBCC_H_
#define GBCC_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBCC_ABI_VERSION 6

typedef enum gbcc_status {
  GBCC_OK = 0,
  GBCC_ERR_INVALID_ARG = 1,  /* bad size, NULL pointer, non-finite input   (InputError)       */
  GBCC_ERR_OOM = 2,          /* device allocation failed                                       */
  GBCC_ERR_CUDA = 3,         /* a CUDA call failed                         (ProgrammingError)  */
  GBCC_ERR_NOT_CONVERGED = 4,/* max_iter reached; results are still written (ccsd.h:469-472)   */
  GBCC_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up                             */
  GBCC_ERR_STATE = 6,        /* call out of order (e.g. residual before set_inputs)            */
  GBCC_ERR_NUMERIC = 7       /* non-finite energy or residual during the iteration             */
} gbcc_status;

typedef enum gbcc_precision {
  GBCC_PREC_FP64 = 0,        /* every contraction in plain FP64                                */
  GBCC_PREC_MIXED = 1,       /* split-BF16 tensor-core contractions, FP64 elsewhere            */
  GBCC_PREC_FP64_TC = 2      /* FP64-grade contractions on the BF16 tensor cores: each operand */
                             /* row in six 8-bit fixed-point slices under its largest         */
                             /* exponent; slice products of one weight summed exactly in FP32,*/
                             /* float-float across chunks (error ~2^-47 of row max x row max) */
} gbcc_precision;

typedef struct gbcc_config {
  int64_t o;                   /* active occupied orbitals                                     */
  int64_t v;                   /* virtual orbitals                                             */
  int32_t precision;           /* gbcc_precision                                               */
  int32_t slices_ladder;       /* BF16 slices per operand, particle-particle ladder (1..3;     */
                               /* 0, the default: chosen from the measured error, see below) */
  int32_t slices_ring;         /* ... o^3 v^3 ring terms and the ladder's T1 part (1..3)       */
  int32_t slices_other;        /* ... every remaining contraction (1..3)                       */
  int32_t refine_iters;        /* FP64-grade iterations after the mixed phase                  */
  double mixed_switch_precision; /* mixed phase ends once converged to this precision;         */
                               /* 0 (default): target_precision                              */
  int32_t max_iter;            /* "max_iter", default 30 (ccsd.h:104)                          */
  double target_precision;     /* Energy precision, default 1e-9 (energy.h:45)                 */
  int32_t diis_start;          /* "diis_start", default 1      (cc/solvers.h:93)               */
  int32_t n_diis;              /* "n_diis", default 8                                          */
  double diis_damp;            /* "diis_damp", default 0                                       */
  int32_t diis_ngroup;         /* "diis_ngroup", default 1                                     */
  int32_t diis_group_nstart;   /* "diis_group_nstart", default 1                               */
  int32_t verbose;             /* print the iteration table (ccsd.h:28-46)                     */
  int32_t device;              /* CUDA device ordinal                                          */
  int32_t use_graphs;          /* 2 (default): gbcc_solve runs the whole loop as one CUDA     */
                               /* graph -- a WHILE node whose body is one iteration, the      */
                               /* convergence test and DIIS bookkeeping decided on the device,*/
                               /* no host synchronisation per iteration; residual calls       */
                               /* replay a graph captured on first use per precision.  1: the */
                               /* same residual graphs with the loop driven from the host     */
                               /* (same decisions and results); 0: direct launches            */
  double slice_tolerance;      /* automatic slices: largest max|dr|/max|r| (r1 and r2) a class */
                               /* may add against 3 slices at the probe amplitudes; 1e-5     */
  int32_t autotune;            /* 1 (default): mixed handles time each tensor-core contraction's */
                               /* candidate tile widths and K splits once and keep the fastest */
  int32_t refine_reset_diis;   /* 1 (default): the DIIS subspace restarts after the update at  */
                               /* the switch to FP64, so the refinement extrapolates with FP64 */
                               /* residuals only (DIISSolver::reset, cc/solvers.h:154-157,     */
                               /* "used when switching to a new solver subspace"); 0: keep it   */
  int32_t refine_precision;    /* precision of the refinement iterations of a mixed handle:    */
                               /* GBCC_PREC_FP64 (default, DFMA) or GBCC_PREC_FP64_TC          */
} gbcc_config;

typedef struct gbcc_inputs {
  const double* eps_o;   /* [o] active occupied orbital energies (diag of the MO Fock)  */
  const double* eps_v;   /* [v] virtual orbital energies                                 */
  const double* Fia;     /* [o][v] */
  const double* Fij;     /* [o][o] */
  const double* Fab;     /* [v][v] */
  const double* Gijab;   /* [o][o][v][v] */
  const double* Gijkl;   /* [o][o][o][o] */
  const double* Giajb;   /* [o][v][o][v] */
  const double* Gijka;   /* [o][o][o][v] */
  const double* Giabc;   /* [o][v][v][v] */
  const double* Gabcd;   /* [v][v][v][v] */
} gbcc_inputs;

/* Density-fitted inputs (the reference's method "df" with the lazy (ab|cd)
 * ladder, ccsd_r1_r2.h:136-184, 309-520): the four-index blocks the DF
 * residual reads plus three-index factors with (pq|rs) = sum_K (K|pq)(K|rs).
 * The (ab|cd) block is never stored: the ladder builds its rows block by
 * block from Xab on the tensor cores every residual, and <ia|bc> is built
 * once from Xai and Xab. */
typedef struct gbcc_df_inputs {
  const double* eps_o;   /* [o] */
  const double* eps_v;   /* [v] */
  const double* Fia;     /* [o][v] */
  const double* Fij;     /* [o][o] */
  const double* Fab;     /* [v][v] */
  const double* Gijab;   /* [o][o][v][v] */
  const double* Gijkl;   /* [o][o][o][o] */
  const double* Giajb;   /* [o][v][o][v] */
  const double* Gijka;   /* [o][o][o][v] */
  int64_t naux;          /* auxiliary (fitting) functions                */
  const double* Xai;     /* [naux][v][o] = (K|ai)  (MPQC's Xai("K,a,i")) */
  const double* Xab;     /* [naux][v][v] = (K|ab)  (MPQC's Xab("K,a,b")) */
} gbcc_df_inputs;

/* Integral-direct inputs (the reference's method "direct",
 * ccsd.h:581-603 and ccsd_r1_r2.h:116-118, 282-286): the MO blocks without
 * Gabcd, plus the AO integrals and the MO coefficients.  The ladder then runs
 * in the AO basis, u(p,r,i,j) = sum_qs (pq|rs) tau_AO(q,s,i,j) with
 * tau_AO = Ca tau Ca^T, and u replaces the (ab|cd) and the Giabc-tau terms. */
typedef struct gbcc_direct_inputs {
  const double* eps_o;   /* [o] */
  const double* eps_v;   /* [v] */
  const double* Fia;     /* [o][v] */
  const double* Fij;     /* [o][o] */
  const double* Fab;     /* [v][v] */
  const double* Gijab;   /* [o][o][v][v] */
  const double* Gijkl;   /* [o][o][o][o] */
  const double* Giajb;   /* [o][v][o][v] */
  const double* Gijka;   /* [o][o][o][v] */
  const double* Giabc;   /* [o][v][v][v] (the ring and T1 terms still read it) */
  int64_t nao;           /* atomic orbitals                                   */
  const double* Gao;     /* [nao][nao][nao][nao] = (pq|rs), chemists' order   */
  const double* Ca;      /* [nao][v] virtual MO coefficients                  */
  const double* Ci;      /* [nao][o] active occupied MO coefficients          */
} gbcc_direct_inputs;

typedef struct gbcc_report {
  int32_t iters;            /* residual evaluations performed                     */
  int32_t converged;        /* 1 if the convergence test of cc/solvers.h:150 held */
  int32_t mixed_iters;      /* of which in mixed precision                        */
  int32_t fp64_iters;       /* of which in plain FP64                             */
  double e_corr;            /* final correlation energy                           */
  double last_dE;
  double last_error;        /* Solver::error of the last residual                 */
  double seconds_total;
  double seconds_residual_mixed;  /* mean seconds per mixed residual              */
  double seconds_residual_fp64;   /* mean seconds per FP64 residual               */
} gbcc_report;

typedef struct gbcc_handle gbcc_handle;

/* Library ABI version (GBCC_ABI_VERSION of the build). */
int gbcc_abi_version(void);

/* Human-readable name of a status code. */
const char* gbcc_status_string(gbcc_status s);

/* Fill *cfg with the reference's defaults (precision FP64, 3/3/3 slices). */
void gbcc_config_default(gbcc_config* cfg);

/* Create a handle on cfg->device.  Replaces the KeyVal constructors. */
gbcc_status gbcc_create(gbcc_handle** out, const gbcc_config* cfg);

/* Copy Fock blocks, orbital energies and MO integrals onto the device and
 * prepare every contraction (split copies of the constant integrals in the
 * mixed mode).  May be called again to replace the inputs. */
gbcc_status gbcc_set_inputs(gbcc_handle* h, const gbcc_inputs* in);

/* Density-fitted alternative to gbcc_set_inputs (host or device pointers):
 * the handle then evaluates the residual of compute_cs_ccsd_r1_df /
 * compute_cs_ccsd_r2_df (ccsd_r1_r2.h:136-184, 309-520) without a v^4
 * array.  The first set call fixes a handle's kind: a handle set up with
 * gbcc_set_inputs rejects this call (GBCC_ERR_STATE) and vice versa, as does
 * a later call with another naux. */
gbcc_status gbcc_set_df_inputs(gbcc_handle* h, const gbcc_df_inputs* in);

/* Integral-direct alternative to gbcc_set_inputs (host or device pointers):
 * the handle evaluates the residual with the U intermediate of the
 * reference's direct method and never holds an MO (ab|cd) array.  The same
 * rule fixes the handle's kind as for gbcc_set_df_inputs. */
gbcc_status gbcc_set_direct_inputs(gbcc_handle* h, const gbcc_direct_inputs* in);

/* Zero-copy alternative to gbcc_set_inputs for integrals too large to hold
 * twice in device memory (the v^4 (ab|cd) block is 84 GB at v = 320):
 * gbcc_device_inputs returns, in *out, device pointers to the handle's own
 * input arrays (writable, same layouts as gbcc_inputs); the caller fills
 * them on the device and then calls gbcc_commit_inputs, which validates the
 * orbital energies and prepares the contractions as gbcc_set_inputs does.
 * The commit gives the (ab|cd) storage back (the residual reads only its
 * pair-symmetric copies): the Gabcd pointer is invalid afterwards, and the
 * next gbcc_device_inputs allocates it again (zeroed).
 * No counterpart in the reference (its integrals live in TiledArray arrays). */
gbcc_status gbcc_device_inputs(gbcc_handle* h, gbcc_inputs* out);
gbcc_status gbcc_commit_inputs(gbcc_handle* h);

/* One residual: tau = t2 + t1 t1, R1 then R2 (R1 sets the FIJ/FAB
 * intermediates R2 reads), in the handle's precision.  t2 must be
 * pair-symmetric, t2(a,b,i,j) = t2(b,a,j,i), as closed-shell CCSD amplitudes
 * are: the particle-particle ladder is evaluated over a <= b, i <= j.  A t2
 * further than 1e-12 max|t2| from that symmetry gives GBCC_ERR_INVALID_ARG. */
gbcc_status gbcc_residual(gbcc_handle* h, const double* t1_ai, const double* t2_abij,
                          double* r1_ai, double* r2_abij);

/* As gbcc_residual with an explicit precision (gbcc_precision).
 * GBCC_PREC_FP64_TC needs a handle whose precision or refine_precision is
 * GBCC_PREC_FP64_TC (its plan and slice packs are built with the inputs);
 * otherwise GBCC_ERR_STATE. */
gbcc_status gbcc_residual_ex(gbcc_handle* h, int32_t precision, const double* t1_ai,
                             const double* t2_abij, double* r1_ai, double* r2_abij);

/* Residual-augmented energy E = 2<f_ai + r1, t1> + <g_abij + r2, 2 tau - tau(b,a,i,j)>
 * and Solver::error = sqrt(|r1|^2 + |r2|^2) / (size(r1) + size(r2)), with FP64
 * deterministic reductions.  Either output pointer may be NULL. */
gbcc_status gbcc_energy(gbcc_handle* h, const double* t1_ai, const double* t2_abij,
                        const double* r1_ai, const double* r2_abij, double* energy,
                        double* error);

/* Allocation-free form of gbcc_energy, for callers that cannot allocate GPU
 * memory when they test convergence: a host framework that owns one fixed
 * device pool and forbids later allocation, or a caller that cannot accept
 * the device-wide synchronisation a cudaMalloc may cause.  It needs no
 * handle: every argument is device memory of the stream's device owned by the
 * caller -- f_ai [v][o], g_abij [v][v][o][o], t1 [v][o], tau [v][v][o][o],
 * r1 [v][o], r2 [v][v][o][o] in, out[0] = energy and out[1] = residual error
 * (as gbcc_energy) written; any other pointer (host memory, another device)
 * gives GBCC_ERR_INVALID_ARG -- and the kernels are enqueued on `stream` (a
 * cudaStream_t; NULL = the legacy default stream) without synchronising.
 * Partial sums go to a fixed 8 MiB __device__ array, so v <= 512 (larger v is
 * rejected with GBCC_ERR_INVALID_ARG).  Calls that overlap on the GPU share
 * that array and race.  The first call on a device (and again in a new CUDA
 * context of it, e.g. after cudaDeviceReset) looks up the array's address;
 * make that first call before any stream capture begins.  No counterpart in
 * the reference. */
gbcc_status gbcc_energy_noalloc(int64_t o, int64_t v, const double* f_ai, const double* g_abij,
                                const double* t1_ai, const double* tau_abij, const double* r1_ai,
                                const double* r2_abij, double* out, void* stream);

/* Full solve from t = 0: Jacobi + DIIS iterations until converged or
 * max_iter.  Writes converged t1/t2 (either may be NULL), E_corr and the
 * report (may be NULL).  Returns GBCC_ERR_NOT_CONVERGED (outputs written) if
 * max_iter was reached, mirroring the reference's warning. */
gbcc_status gbcc_solve(gbcc_handle* h, double* t1_ai, double* t2_abij, double* e_corr,
                       gbcc_report* report);

/* Many independent solves at once (e.g. the clusters of a batch): gbcc_solve
 * of every handle, each from its own host thread, so that all the solves --
 * each one CUDA graph on its handle's stream, stopping by its own
 * convergence test on the device -- are in flight on the GPU together.
 * e_corr[k], reports[k] and statuses[k] (any of the arrays may be NULL)
 * receive handle k's results and gbcc_solve status.  Returns the first
 * failing status in handle order (its message in gbcc_last_error of that
 * handle), else GBCC_ERR_NOT_CONVERGED if a solve hit max_iter, else GBCC_OK.
 * A handle may appear once.  The reference solves one molecule at a time
 * (ccsd.h:367-468); no counterpart. */
gbcc_status gbcc_solve_batch(gbcc_handle* const* handles, int32_t count, double* e_corr, gbcc_report* reports,
                             gbcc_status* statuses);

/* Perturbative triples correction (T) of closed-shell CCSD: the reference's
 * CCSD_T::compute_ccsd_t (src/mpqc/chemistry/qc/lcao/cc/ccsd_t.h:143-172)
 * with its "straight" approach (:1127-1167, denominators :2274-2333), from
 * t1/t2 (host or device pointers in gbcc_residual's layouts; NULL: the
 * amplitudes of the handle's last gbcc_solve) and the handle's <ij|ab>,
 * <ij|ka>, <ia|bc> and orbital energies.  precision (gbcc_precision) sets the
 * arithmetic of the o^3 v^4 contractions -- GBCC_PREC_FP64, MIXED (three
 * BF16 slices) or FP64_TC; the energy sums are FP64.  *e_t receives E(T);
 * the CCSD(T) energy is the CCSD energy plus E(T) (ccsd_t.h:183-195). */
gbcc_status gbcc_triples(gbcc_handle* h, int32_t precision, const double* t1_ai, const double* t2_abij,
                         double* e_t);

/* Release the handle and all its device memory.  NULL is accepted. */
gbcc_status gbcc_destroy(gbcc_handle* h);

/* Amplitudes the next gbcc_solve starts from instead of t = 0 (host or
 * device pointers, t1[a][i], t2[a][b][i][j], t2 pair-symmetric): a restart.
 * Counterpart of CCSD::set_t1 / set_t2 (ccsd.h:183-185), which store
 * amplitudes in the wavefunction; here they seed one solve and are then
 * consumed. */
gbcc_status gbcc_set_amplitudes(gbcc_handle* h, const double* t1_ai, const double* t2_abij);

/* Checkpoint of the amplitudes of the last gbcc_solve on this handle: a file
 * of the 8 bytes "GBCCAMP1", int64 o, int64 v, double E_corr, then t1 and t2
 * as FP64 in host byte order.  GBCC_ERR_STATE if no solve has completed since
 * the inputs were set (or a residual / energy call has replaced the
 * amplitudes).  No reference counterpart (MPQC keeps T1/T2 in memory only). */
gbcc_status gbcc_save_amplitudes(gbcc_handle* h, const char* path);

/* Read a checkpoint written by gbcc_save_amplitudes (same o and v) and seed
 * the next gbcc_solve with it, as gbcc_set_amplitudes does; *e_corr (may be
 * NULL) receives the energy stored with it. */
gbcc_status gbcc_load_amplitudes(gbcc_handle* h, const char* path, double* e_corr);

/* Slice counts in use per contraction class {ladder, ring, other} once inputs
 * are set, and for classes configured as 0 the measured max|dr|/max|r| of the
 * chosen count against 3 slices (-1: fixed by the configuration).  In mixed
 * mode gbcc_set_inputs / gbcc_commit_inputs choose them: at probe amplitudes
 * (two Jacobi steps from t = 0) each automatic class takes the fewest slices
 * (3, 2 or 1) whose residual change stays within slice_tolerance.  No
 * reference counterpart (MPQC computes in FP64 only). */
gbcc_status gbcc_slice_policy(gbcc_handle* h, int32_t slices[3], double rel_change[3]);

/* Re-choose the automatic slice counts (mixed handles) at the caller's
 * amplitudes t1[v][o], t2[v][v][o][o] (host or device) instead of the probe
 * amplitudes gbcc_set_inputs used, e.g. before evaluating residuals at given
 * amplitudes with gbcc_residual.  Same rule as above; leaves t = 0 in the
 * handle.  No reference counterpart. */
/* The autotune table (config autotune): every tensor-core contraction timed
 * by any handle of the process is recorded by shape (SM count, term class,
 * M x N x K, slice count, output orientation), and handles created later take
 * the recorded tile untimed.  gbcc_autotune_save writes the table as text;
 * gbcc_autotune_load merges a file written by gbcc_autotune_save
 * (GBCC_ERR_INVALID_ARG, table unchanged, if it cannot be read or is
 * malformed); gbcc_autotune_clear empties it.  No counterpart in the
 * reference (TiledArray picks no tiles at run time). */
gbcc_status gbcc_autotune_save(const char* path);
gbcc_status gbcc_autotune_load(const char* path);
gbcc_status gbcc_autotune_clear(void);

/* Layout adapters for a caller whose tensors are tiled (MPQC's TiledArray
 * arrays over TiledRange1 boundaries, e.g. the uneven occupied / virtual
 * tilings of src/mpqc/chemistry/qc/lcao/expression/trange1_engine.cpp:10-20):
 * `tiles` holds every tile of a rank-`rank` array one after another, in
 * row-major order over the tile grid, each tile row-major over its own
 * extents; `dense` is the row-major array the entry points above take.
 * bounds[d] lists the nbounds[d] boundaries of dimension d (0 = b0 < b1 <
 * ... < extent).  Host memory, no GPU; GBCC_ERR_INVALID_ARG for rank outside
 * 1..8, missing or non-increasing boundaries, or NULL arrays.  The residual
 * does not depend on the tiling: a caller converts its inputs once and its
 * amplitudes at the call. */
gbcc_status gbcc_tiles_to_dense(int32_t rank, const int64_t* const* bounds, const int32_t* nbounds,
                                const double* tiles, double* dense);
gbcc_status gbcc_dense_to_tiles(int32_t rank, const int64_t* const* bounds, const int32_t* nbounds,
                                const double* dense, double* tiles);

gbcc_status gbcc_calibrate_slices(gbcc_handle* h, const double* t1_ai, const double* t2_abij);

/* Message of the last failing call on this handle ("" if none); with a NULL
 * handle, the message of the last failed gbcc_create on this thread. */
const char* gbcc_last_error(const gbcc_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* GBCC_H_ */
