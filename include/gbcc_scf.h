/*
 * gbcc_scf.h -- C ABI of the input producer of the CCSD solver: AO integrals,
 * closed-shell RHF and the AO -> MO transform into the CCSD handle, on the GPU.
 *
 * MPQC builds the CCSD inputs with Libint2 integrals, its RHF and the LCAO
 * factory (paths relative to the MPQC source tree):
 *
 *   gbcc_scf_create     <- the basis and molecule set-up of AOWavefunction and
 *                          the AO integrals of the factory (one-body: S, T, V;
 *                          two-body (mu nu|la si))
 *                                          src/mpqc/chemistry/qc/lcao/basis/basis.cpp:28,49
 *                                          src/mpqc/chemistry/qc/lcao/integrals/make_engine.h:24-88
 *   gbcc_scf_run        <- RHF::solve      src/mpqc/chemistry/qc/lcao/scf/rhf_impl.h:178-262
 *                          (keywords of RHF(const KeyVal&), rhf.h and rhf.cpp:10-44)
 *   gbcc_scf_orbitals   <- the canonical orbital space and its energies
 *                                          src/mpqc/chemistry/qc/lcao/scf/mo_build.h:19-26, 353-393
 *   gbcc_scf_ccsd_inputs<- LCAOFactory::compute4 of the CCSD integral blocks and
 *                          make_diagonal_fpq, with frozen core as init_sdref
 *                                          src/mpqc/chemistry/qc/lcao/factory/lcao_factory.h:378-509
 *                                          src/mpqc/chemistry/qc/lcao/cc/ccsd.h:218-229, 281-322
 *                                          src/mpqc/chemistry/qc/lcao/wfn/lcao_wfn.h:97-190
 *
 * Integrals are computed over contracted Gaussians with s, p and d shells by
 * the McMurchie-Davidson scheme, in FP64, and every basis function is scaled
 * to unit self-overlap.  The full (mu nu|la si) array stays in device memory
 * (N^4 doubles: 26.5 GB at N = 240) for the Fock builds and the transform.
 *
 * Conventions as in gbcc.h: every call returns a gbcc_status, host arrays are
 * owned by the caller, gbcc_last_scf_error() gives the last failure's message.
 */
#ifndef GBCC_SCF_H_
#define GBCC_SCF_H_

#include <stdint.h>

#include "gbcc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbcc_molecule {
  int32_t natom;
  const double* charge;  /* [natom] nuclear charges Z                              */
  const double* xyz;     /* [natom][3] nuclear positions, Bohr                     */
  int32_t mol_charge;    /* molecular charge; the electron count must be even      */
} gbcc_molecule;

typedef struct gbcc_basis {
  int32_t nshell;
  const int32_t* atom;   /* [nshell] atom of each shell (its centre)               */
  const int32_t* l;      /* [nshell] angular momentum, 0..2                        */
  const int32_t* nprim;  /* [nshell] primitives per shell                          */
  const double* exps;    /* [sum nprim] exponents                                  */
  const double* coefs;   /* [sum nprim] contraction coefficients of normalised     */
                         /* primitives, as basis-set libraries list them           */
  int32_t pure;          /* 1: spherical d shells (5 functions: xy, yz, z2, xz,    */
                         /* x2-y2), 0: Cartesian (6: xx, xy, xz, yy, yz, zz)       */
} gbcc_basis;

typedef struct gbcc_scf_config {
  int32_t device;        /* CUDA device ordinal                                    */
  int32_t max_iter;      /* "max_iter" of RHF, default 30                          */
  double threshold;      /* energy change and |FDS - SDF|_F / N^2 limit, 1e-11     */
  int32_t n_diis;        /* Fock DIIS subspace, default 8                          */
  int32_t verbose;       /* print the iteration lines                              */
} gbcc_scf_config;

typedef struct gbcc_scf_report {
  int32_t nbf;           /* basis functions                                        */
  int32_t nocc;          /* doubly occupied orbitals                               */
  int32_t iters;
  int32_t converged;
  double energy;         /* E_RHF including the nuclear repulsion                  */
  double e_nuc;
  double seconds_one_body;
  double seconds_eri;
  double seconds_scf;
  double seconds_transform;  /* last gbcc_scf_ccsd_inputs                          */
} gbcc_scf_report;

typedef struct gbcc_scf gbcc_scf;

void gbcc_scf_config_default(gbcc_scf_config* cfg);

/* Validate the molecule and basis, compute S, H = T + V and (mu nu|la si) on
 * the device.  No reference counterpart as one call (see the table above). */
gbcc_status gbcc_scf_create(gbcc_scf** out, const gbcc_molecule* mol, const gbcc_basis* basis,
                            const gbcc_scf_config* cfg);

/* Closed-shell RHF from the core-Hamiltonian guess: Fock builds on the device,
 * DIIS on F with the gradient FDS - SDF, until |dE| <= threshold and
 * |FDS - SDF|_F / N^2 <= threshold.  GBCC_ERR_NOT_CONVERGED at max_iter (the
 * reference throws MaxIterExceeded). */
gbcc_status gbcc_scf_run(gbcc_scf* h, gbcc_scf_report* report);

/* AO matrices in the normalised basis: S, H [N][N] and, if G is not NULL,
 * (mu nu|la si) [N][N][N][N] (any pointer may be NULL). */
gbcc_status gbcc_scf_ao(gbcc_scf* h, double* S, double* H, double* G);

/* Canonical orbitals after gbcc_scf_run: C [N][N] (column p = orbital p,
 * ascending energies) and eps [N] (either may be NULL). */
gbcc_status gbcc_scf_orbitals(gbcc_scf* h, double* C, double* eps);

/* Transform (mu nu|la si) to the MO basis on the device and write the CCSD
 * inputs of the standard method -- orbital energies, Fock blocks and the six
 * <pq|rs> blocks in MPQC annotation order, with the lowest n_frozen occupied
 * orbitals frozen -- straight into the device inputs of `cc`, then commit
 * them (gbcc_device_inputs + gbcc_commit_inputs).  cc must have been created
 * with o = nocc - n_frozen and v = N - nocc on the same device. */
gbcc_status gbcc_scf_ccsd_inputs(gbcc_scf* h, int32_t n_frozen, gbcc_handle* cc);

/* Release the handle and its device memory; NULL is accepted. */
gbcc_status gbcc_scf_destroy(gbcc_scf* h);

/* Message of the last failing call on this handle, or with NULL of the last
 * failed gbcc_scf_create on this thread. */
const char* gbcc_last_scf_error(const gbcc_scf* h);

#ifdef __cplusplus
}
#endif

#endif /* GBCC_SCF_H_ */
