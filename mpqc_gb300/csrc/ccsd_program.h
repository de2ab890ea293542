// The CCSD residual program and the device tensors it works on.
#pragma once

#include <memory>
#include <vector>

#include "engine.h"
#include "kernels.h"

namespace gbcc {

struct CcsdTensors {
  // inputs (constant after set_inputs), MPQC annotation order
  Tensor *Fia, *Fij, *Fab, *Gijab, *Gijkl, *Giajb, *Gijka, *Giabc, *Gabcd, *eps_o, *eps_v;
  Tensor *f_ai, *g_abij;  // Fia("i,a") as (a,i); Gijab("i,j,a,b") as (a,b,i,j)
  Tensor *Dinv1, *Dinv2;  // reciprocal Jacobi denominators [v][o], [v][v][o][o]
  // amplitudes and residuals
  Tensor *t1, *t2, *tau, *r1, *r2;
  // intermediates
  // (P = 2 j - k of the ring terms, k = K)
  Tensor *tki, *FAB, *FIJ, *hkc, *r2u, *Y1, *Y2, *gki, *gac, *P, *K, *tmp, *W, *tmp2;
  // K(k,a,k,c) and P(a,k,k,c) before their Giabc t1 terms (g_ac reads the increments)
  Tensor *diagK, *diagP;
  // particle-particle ladder over pair-(anti)symmetric combinations: G+/G- of
  // Gabcd over (a <= b) x (c <= d) and of Giabc over (k a) x (c <= d)
  // (constants), tau+/tau- over (c <= d) x (i <= j), and the pair products
  Tensor *Gp, *Gm, *Gip, *Gim, *taup, *taum, *Bp, *Bm, *Xp, *Xm;
  // hole-hole ladder over pair combinations (kernels.cu): Gijab's pair
  // factors over (k <= l) x (c <= d) (constants) and W+- over (k <= l) x (i <= j)
  Tensor *Gtp = nullptr, *Gtm = nullptr, *Wt = nullptr, *Wm = nullptr;
  // density-fitted inputs (naux > 0): three-index factors in MPQC order
  // Xai[K][a][i] = (K|ai), Xab[K][a][b] = (K|ab) instead of Giabc / Gabcd;
  // Giabc is built from them on the device, (ab|cd) never exists whole: the
  // ladder builds G+- rows one block of a at a time from Xac[a][c][K]
  int64_t naux = 0;
  Tensor *Xai = nullptr, *Xab = nullptr, *Xac = nullptr;
  struct DfBlock {
    int64_t a0, a1, rows_p, rows_m;
    // views: Xac rows a of the block, Xac rows b >= a0, Gblk[a - a0][b - a0][c][d],
    // its G+- rows and the B+- rows of the block
    Tensor xa, xb, g, gp, gm, bp, bm;
  };
  std::vector<std::unique_ptr<DfBlock>> df_blocks;
  // integral-direct inputs (nao > 0, the reference's method "direct"): AO
  // integrals (pq|rs) and MO coefficients instead of Gabcd.  The ladder runs
  // in the AO basis, u(p,r,i,j) = sum_qs (pq|rs) tau_AO(q,s,i,j), and its MO
  // images replace the (ab|cd) and the Giabc-tau terms
  int64_t nao = 0;
  Tensor *Gao = nullptr, *Ca = nullptr, *Ci = nullptr, *Gpao = nullptr, *Gmao = nullptr;
  Tensor *Xq = nullptr, *tauao = nullptr, *tauaop = nullptr, *tauaom = nullptr, *Bpao = nullptr, *Bmao = nullptr;
  Tensor *u = nullptr, *U1 = nullptr, *U2 = nullptr;
  void create(Engine& E, int64_t o, int64_t v, int64_t naux_df = 0, int64_t nao_direct = 0);
};

void setup_program(Engine& E, const CcsdTensors& S);
void residual_program(Engine& E, const CcsdTensors& S);

}  // namespace gbcc
