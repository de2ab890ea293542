// The CCSD residual program and the device tensors it works on.
#pragma once

#include "engine.h"
#include "kernels.h"

namespace gbcc {

struct CcsdTensors {
  // inputs (constant after set_inputs), MPQC annotation order
  Tensor *Fia, *Fij, *Fab, *Gijab, *Gijkl, *Giajb, *Gijka, *Giabc, *Gabcd, *eps_o, *eps_v;
  Tensor *f_ai, *g_abij;  // Fia("i,a") as (a,i); Gijab("i,j,a,b") as (a,b,i,j)
  // amplitudes and residuals
  Tensor *t1, *t2, *tau, *r1, *r2;
  // intermediates
  Tensor *tki, *FAB, *FIJ, *hkc, *r2u, *Y1, *Y2, *gki, *gac, *J, *K, *tmp, *W, *tmp2;
  // particle-particle ladder over pair-(anti)symmetric combinations: G+/G- of
  // Gabcd over (a <= b) x (c <= d) and of Giabc over (k a) x (c <= d)
  // (constants), tau+/tau- over (c <= d) x (i <= j), and the pair products
  Tensor *Gp, *Gm, *Gip, *Gim, *taup, *taum, *Bp, *Bm, *Xp, *Xm;
  void create(Engine& E, int64_t o, int64_t v);
};

void setup_program(Engine& E, const CcsdTensors& S);
void residual_program(Engine& E, const CcsdTensors& S);

}  // namespace gbcc
