// The closed-shell CCSD residual as a program of engine operations.
//
// One statement per einstein-index expression of the reference (paths
// relative to the MPQC source tree):
//   compute_cs_ccsd_r1  src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:70-124
//   compute_cs_ccsd_r2  src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:198-293
//   intermediates       src/mpqc/chemistry/qc/lcao/cc/ccsd_intermediates.h:57-193
// Tensor storage follows the MPQC annotation order (t1[a][i], t2[a][b][i][j],
// Gijab[i][j][a][b], ...); a label string names the stored dimensions in
// order, so Giabc("kadc") is <k a|d c> stored as Giabc[k][a][d][c].
//
// Some expressions are regrouped; each is an exact rearrangement of the same
// sums:
//  - no o v^3 temporary: the reference's (Giabc(i,c,a,b) - Giajb(k,b,i,c)
//    t1(a,k)) t1(c,j) is Giabc(i,c,a,b) t1(c,j) - (Giajb(k,b,i,c) t1(c,j))
//    t1(a,k), and (Gijka(j,i,k,a) + Gijab(i,k,a,c) t1(c,j)) t1(b,k) two
//    products;
//  - r2 = r2u(a,b,i,j) + r2u(b,a,j,i) + ..., so a term X(a,b,i,j) of r2u may be
//    replaced by X(b,a,j,i).  Done for -Y1(k,b,i,j) t1(a,k), and the ladder's
//    -tmp2(k,a,j,i) t1(b,k) - tmp2(k,b,i,j) t1(a,k) of r2 becomes one term of
//    r2u: the four products with t1(b,k) form one contraction;
//  - r1's (2 Giabc(k,a,c,d) - Giabc(k,a,d,c)) tau(c,d,k,i) is read off tmp2
//    (tau(c,d,k,i) = tau(d,c,i,k) for pair-symmetric amplitudes), so tmp2 is
//    evaluated first;
//  - h_kc(k,c) (2 t2(c,a,k,i) - t2(c,a,i,k) + t1(c,i) t1(a,k)) is not
//    materialised: the t1 t1 part is t1(a,k) (h_kc(k,c) t1(c,i));
//  - nor is T(d,a,i,l) = 0.5 t2(d,a,i,l) + t1(d,i) t1(a,l): the ring
//    contractions pack its two terms directly;
//  - g_ac's sum_kd (2 Giabc(k,a,d,c) - Giabc(k,a,c,d)) t1(d,k) is read off the
//    diagonals i = k of K's and P's Giabc t1 terms (their increments, kernels.cu);
//  - the hole-hole ladder W(k,l,i,j) tau(a,b,k,l) runs as pair products over
//    k <= l and i <= j (like the particle-particle ladder, kernels.cu), and
//    adds to that ladder's B+-; one pass then writes r2: r2u(a,b,i,j) +
//    r2u(b,a,j,i) with the tmp terms folded in (-0.5 tmp(a,b,i,j) -
//    tmp(b,a,i,j) of r2u and their images), g_abij and the unpacked B+-
//    (integral-direct: W and r2 = W tau as written, the pass adds to r2).
#include "ccsd_program.h"

namespace gbcc {

namespace {

// a tensor whose storage lies inside another allocation
Tensor view(const std::string& name, double* d, std::initializer_list<int64_t> dims) {
  Tensor t;
  t.name = name;
  t.d = d;
  t.rank = static_cast<int>(dims.size());
  int k = 0;
  for (int64_t x : dims) t.dim[k++] = x;
  return t;
}

int64_t pairs_before(int64_t a, int64_t v) { return a * v - a * (a - 1) / 2; }     // sym pairs with first < a
int64_t anti_before(int64_t a, int64_t v) { return a * (v - 1) - a * (a - 1) / 2; }  // anti pairs with first < a

}  // namespace

// rows a per block of the density-fitted ladder for handles set up from now
// on (0: the default, Gblk of at most 4 GB); a test hook
int64_t g_df_block_rows = 0;

void CcsdTensors::create(Engine& E, int64_t o, int64_t v, int64_t naux_df, int64_t nao_direct) {
  naux = naux_df;
  nao = nao_direct;
  const bool mo_ladder = naux == 0 && nao == 0;
  Fia = &E.tensor("Fia", {o, v}, true);
  Fij = &E.tensor("Fij", {o, o}, true);
  Fab = &E.tensor("Fab", {v, v}, true);
  Gijab = &E.tensor("Gijab", {o, o, v, v}, true);
  Gijkl = &E.tensor("Gijkl", {o, o, o, o}, true);
  Giajb = &E.tensor("Giajb", {o, v, o, v}, true);
  Gijka = &E.tensor("Gijka", {o, o, o, v}, true);
  Giabc = &E.tensor("Giabc", {o, v, v, v}, true);
  Gabcd = mo_ladder ? &E.tensor("Gabcd", {v, v, v, v}, true) : nullptr;
  eps_o = &E.tensor("eps_o", {o}, true);
  eps_v = &E.tensor("eps_v", {v}, true);
  f_ai = &E.tensor("f_ai", {v, o}, true);
  g_abij = &E.tensor("g_abij", {v, v, o, o}, true);
  Dinv1 = &E.tensor("Dinv1", {v, o}, true);
  Dinv2 = &E.tensor("Dinv2", {v, v, o, o}, true);
  t1 = &E.tensor("t1", {v, o});
  t2 = &E.tensor("t2", {v, v, o, o});
  tau = &E.tensor("tau", {v, v, o, o});
  r1 = &E.tensor("r1", {v, o});
  r2 = &E.tensor("r2", {v, v, o, o});
  tki = &E.tensor("tki", {o, o});
  FAB = &E.tensor("FAB", {v, v});
  FIJ = &E.tensor("FIJ", {o, o});
  hkc = &E.tensor("hkc", {o, v});
  r2u = &E.tensor("r2u", {v, v, o, o});
  Y1 = &E.tensor("Y1", {o, v, o, o});
  Y2 = &E.tensor("Y2", {o, o, v, o});
  gki = &E.tensor("gki", {o, o});
  gac = &E.tensor("gac", {v, v});
  diagK = &E.tensor("diagK", {o, v, v});
  diagP = &E.tensor("diagP", {o, v, v});
  P = &E.tensor("P", {v, o, o, v});
  K = &E.tensor("K", {o, v, o, v});
  tmp = &E.tensor("tmp", {v, v, o, o});
  W = &E.tensor("W", {o, o, o, o});
  tmp2 = &E.tensor("tmp2", {o, v, o, o});
  const int64_t np = v * (v + 1) / 2, nm = v * (v - 1) / 2, sp = o * (o + 1) / 2, sm = o * (o - 1) / 2;
  Gp = mo_ladder ? &E.tensor("Gp", {np, np}, true) : nullptr;
  Gm = mo_ladder ? &E.tensor("Gm", {nm, nm}, true) : nullptr;
  if (nao > 0) {
    // the AO ladder replaces both MO pair ladders (G+- of Gabcd and of Giabc)
    const int64_t n = nao, npa = n * (n + 1) / 2, nma = n * (n - 1) / 2;
    Gao = &E.tensor("Gao", {n, n, n, n}, true);
    Ca = &E.tensor("Ca", {n, v}, true);
    Ci = &E.tensor("Ci", {n, o}, true);
    Gpao = &E.tensor("Gpao", {npa, npa}, true);
    Gmao = &E.tensor("Gmao", {nma, nma}, true);
    Xq = &E.tensor("Xq", {n, v, o, o});
    tauao = &E.tensor("tauao", {n, n, o, o});
    tauaop = &E.tensor("tauaop", {npa, sp});
    tauaom = &E.tensor("tauaom", {nma, sm});
    Bpao = &E.tensor("Bpao", {npa, sp});
    Bmao = &E.tensor("Bmao", {nma, sm});
    u = &E.tensor("u", {n, n, o, o});
    U1 = &E.tensor("U1", {v, n, o, o});
    U2 = &E.tensor("U2", {o, n, o, o});
    return;
  }
  Gip = &E.tensor("Gip", {o * v, np}, true);
  Gim = &E.tensor("Gim", {o * v, nm}, true);
  taup = &E.tensor("taup", {np, sp});
  taum = &E.tensor("taum", {nm, sm});
  Bp = &E.tensor("Bp", {np, sp});
  Bm = &E.tensor("Bm", {nm, std::max<int64_t>(sm, 1)});
  Xp = &E.tensor("Xp", {o * v, sp});
  Xm = &E.tensor("Xm", {o * v, sm});
  Gtp = &E.tensor("Gtp", {sp, np}, true);
  Gtm = &E.tensor("Gtm", {std::max<int64_t>(sm, 1), std::max<int64_t>(nm, 1)}, true);
  Wt = &E.tensor("Wt", {sp, sp});
  Wm = &E.tensor("Wm", {std::max<int64_t>(sm, 1), std::max<int64_t>(sm, 1)});
  if (naux > 0) {
    Xai = &E.tensor("Xai", {naux, v, o}, true);
    Xab = &E.tensor("Xab", {naux, v, v}, true);
    Xac = &E.tensor("Xac", {v, v, naux});
    // blocks of a: Gblk[a - a0][b][c][d] of at most ~4 GB
    int64_t blk = std::max<int64_t>(1, std::min<int64_t>(v, (int64_t{1} << 29) / std::max<int64_t>(1, v * v * v)));
    if (g_df_block_rows > 0) blk = std::min(v, g_df_block_rows);
    const int64_t rows_p_max = pairs_before(blk, v), rows_m_max = std::max<int64_t>(1, anti_before(blk, v));
    Tensor& gblk = E.tensor("df_gblk", {blk, v, v, v});
    Tensor& gpb = E.tensor("df_gp", {rows_p_max, np});
    Tensor& gmb = E.tensor("df_gm", {rows_m_max, std::max<int64_t>(nm, 1)});
    df_blocks.clear();
    for (int64_t a0 = 0; a0 < v; a0 += blk) {
      auto b = std::make_unique<DfBlock>();
      const int64_t a1 = std::min(v, a0 + blk), n = a1 - a0;
      b->a0 = a0;
      b->a1 = a1;
      b->rows_p = pairs_before(a1, v) - pairs_before(a0, v);
      b->rows_m = anti_before(a1, v) - anti_before(a0, v);
      const std::string tag = "@" + std::to_string(a0);
      b->xa = view("Xac" + tag, Xac->d + a0 * v * naux, {n, v, naux});
      b->xb = view("Xac>" + tag, Xac->d + a0 * v * naux, {v - a0, v, naux});
      b->g = view("df_gblk" + tag, gblk.d, {n, v - a0, v, v});
      b->gp = view("df_gp" + tag, gpb.d, {b->rows_p, np});
      b->gm = view("df_gm" + tag, gmb.d, {std::max<int64_t>(b->rows_m, 1), std::max<int64_t>(nm, 1)});
      b->bp = view("Bp" + tag, Bp->d + pairs_before(a0, v) * sp, {b->rows_p, sp});
      b->bm = view("Bm" + tag, Bm->d + anti_before(a0, v) * std::max<int64_t>(sm, 1),
                   {std::max<int64_t>(b->rows_m, 1), std::max<int64_t>(sm, 1)});
      df_blocks.push_back(std::move(b));
    }
  }
}

// f_ai(a,i) = Fia(i,a), g_abij(a,b,i,j) = Gijab(i,j,a,b)  (ccsd.h:325-330); the
// reciprocal Jacobi denominators;
// G+/G- of Gabcd and Giabc for the pair-symmetric ladder (kernels.cu)
void setup_program(Engine& E, const CcsdTensors& S) {
  E.assign(ix(*S.f_ai, "ai"), 0.0, {f1(1.0, ix(*S.Fia, "ia"))});
  E.assign(ix(*S.g_abij, "abij"), 0.0, {f1(1.0, ix(*S.Gijab, "ijab"))});
  const int64_t v = S.t1->dim[0], o = S.t1->dim[1];
  {
    const double *eo = S.eps_o->d, *ev = S.eps_v->d;
    double *d1 = S.Dinv1->d, *d2 = S.Dinv2->d;
    E.custom([=](cudaStream_t st) { launch_denominators(o, v, eo, ev, d1, d2, st); }, 1);
  }
  if (S.nao > 0) {
    const int64_t n = S.nao;
    const double* Gao = S.Gao->d;
    double *Gp = S.Gpao->d, *Gm = S.Gmao->d;
    E.custom([=](cudaStream_t st) { launch_build_gpm_chem(n, Gao, Gp, Gm, st); }, 1);
    return;
  }
  if (S.naux > 0) {
    // density fitting: Xac(a,c,K) = Xab(K,a,c); <ia|bc> = (ib|ac) = sum_K Xai(K,b,i) Xab(K,a,c)
    E.assign(ix(*S.Xac, "acK"), 0.0, {f1(1.0, ix(*S.Xab, "Kac"))});
    E.contract(ix(*S.Giabc, "iabc"), 0.0, 1.0, {{1.0, ix(*S.Xai, "Kbi")}}, {{1.0, ix(*S.Xab, "Kac")}}, kClassOther);
  } else {
    const double* Gabcd = S.Gabcd->d;
    double *Gp = S.Gp->d, *Gm = S.Gm->d;
    E.custom([=](cudaStream_t st) { launch_build_gpm(v, v, true, Gabcd, Gp, Gm, st); }, 1);
  }
  const double* Giabc = S.Giabc->d;
  double *Gip = S.Gip->d, *Gim = S.Gim->d;
  E.custom([=](cudaStream_t st) { launch_build_gpm(o, v, false, Giabc, Gip, Gim, st); }, 1);
  const double* Gijab = S.Gijab->d;
  double *Gtp = S.Gtp->d, *Gtm = (o > 1 && v > 1) ? S.Gtm->d : nullptr;
  E.custom([=](cudaStream_t st) { launch_build_gpm_oo(o, v, Gijab, Gtp, Gtm, st); }, 1);
}

void residual_program(Engine& E, const CcsdTensors& S) {
  const Tensor &Fia = *S.Fia, &Fij = *S.Fij, &Fab = *S.Fab, &Gijab = *S.Gijab, &Gijkl = *S.Gijkl,
               &Giajb = *S.Giajb, &Gijka = *S.Gijka, &Giabc = *S.Giabc;
  const Tensor &t1 = *S.t1, &t2 = *S.t2, &tau = *S.tau;
  const Tensor &r1 = *S.r1, &r2 = *S.r2;
  const TermClass O = kClassOther, R = kClassRing, L = kClassLadder;
  const int64_t v = t1.dim[0], o = t1.dim[1];
  const bool minus = v > 1 && o > 1;  // otherwise the antisymmetric pair parts are empty
  const double* tau_d = tau.d;
  double *r1d = r1.d, *r2d = r2.d, *tmp2 = S.tmp2->d;
  const bool direct = S.nao > 0;

  if (direct) {
    // integral-direct (ccsd.h:581-603): tau_AO(q,s,i,j) = Ca(q,a) tau(a,b,i,j) Ca(s,b)
    // and u(p,r,i,j) = (pq|rs) tau_AO(q,s,i,j) over AO pairs p <= r, q <= s
    // (the pair-symmetric ladder of the standard method on the AO tensor);
    // tmp2(k,a,i,j) = Ci(p,k) u(p,r,i,j) Ca(r,a) equals Giabc(k,a,c,d) tau(c,d,i,j)
    const int64_t n = S.nao;
    const bool minus_ao = n > 1 && o > 1;
    const Tensor &Ca = *S.Ca, &Ci = *S.Ci, &u = *S.u;
    E.contract(ix(*S.Xq, "qbij"), 0.0, 1.0, {{1.0, ix(Ca, "qa")}}, {{1.0, ix(tau, "abij")}}, O);
    E.contract(ix(*S.tauao, "qsij"), 0.0, 1.0, {{1.0, ix(*S.Xq, "qbij")}}, {{1.0, ix(Ca, "sb")}}, O);
    const double* tao = S.tauao->d;
    double *tp = S.tauaop->d, *tm = S.tauaom->d, *bp = S.Bpao->d, *bm = S.Bmao->d, *ud = u.d;
    E.custom([=](cudaStream_t st) { launch_tau_pm(o, n, tao, tp, tm, st); }, 1);
    E.contract(ix(*S.Bpao, "PS"), 0.0, 1.0, {{1.0, ix(*S.Gpao, "PQ")}}, {{1.0, ix(*S.tauaop, "QS")}}, L);
    if (minus_ao)
      E.contract(ix(*S.Bmao, "XZ"), 0.0, 1.0, {{1.0, ix(*S.Gmao, "XY")}}, {{1.0, ix(*S.tauaom, "YZ")}}, L);
    E.custom([=](cudaStream_t st) { launch_pair_unpack(n, n, o, true, bp, minus_ao ? bm : nullptr, 0.0, ud, st); },
             1);
    E.contract(ix(*S.U2, "krij"), 0.0, 1.0, {{1.0, ix(Ci, "pk")}}, {{1.0, ix(u, "prij")}}, O);
    E.contract(ix(*S.tmp2, "kaij"), 0.0, 1.0, {{1.0, ix(*S.U2, "krij")}}, {{1.0, ix(Ca, "ra")}}, O);
  } else {
    // tmp2(k,a,i,j) = Giabc(k,a,c,d) tau(c,d,i,j) (ccsd_r1_r2.h:277) as sums over
    // c <= d of the pair-(anti)symmetric combinations (kernels.cu), unpacked
    double *taup = S.taup->d, *taum = S.taum->d, *Xp = S.Xp->d, *Xm = S.Xm->d;
    E.custom([=](cudaStream_t st) { launch_tau_pm(o, v, tau_d, taup, taum, st); }, 1);
    E.contract(ix(*S.Xp, "RS"), 0.0, 1.0, {{1.0, ix(*S.Gip, "RQ")}}, {{1.0, ix(*S.taup, "QS")}}, R);
    if (minus) E.contract(ix(*S.Xm, "RZ"), 0.0, 1.0, {{1.0, ix(*S.Gim, "RY")}}, {{1.0, ix(*S.taum, "YZ")}}, R);
    E.custom([=](cudaStream_t st) { launch_pair_unpack(o, v, o, false, Xp, minus ? Xm : nullptr, 0.0, tmp2, st); },
             1);
  }

  // ----- R1 (ccsd_r1_r2.h:70-124) -----
  // r1(a,i) = Fia(i,a) - 2 (Fia(k,c) t1(c,i)) t1(a,k)
  E.contract(ix(*S.tki, "ki"), 0.0, 1.0, {{1.0, ix(Fia, "kc")}}, {{1.0, ix(t1, "ci")}}, O);
  E.assign(ix(r1, "ai"), 0.0, {f1(1.0, ix(Fia, "ia"))});
  E.contract(ix(r1, "ai"), 1.0, -2.0, {{1.0, ix(*S.tki, "ki")}}, {{1.0, ix(t1, "ak")}}, O);
  // h_ac = F_vv(Fab, gbar, tau); FAB = h_ac; r1 += h_ac(a,c) t1(c,i)
  // gbar(k,l,c,d) = 2 Gijab(k,l,c,d) - Gijab(l,k,c,d)
  E.assign(ix(*S.FAB, "ac"), 0.0, {f1(1.0, ix(Fab, "ac"))});
  E.contract(ix(*S.FAB, "ac"), 1.0, -1.0, {{2.0, ix(Gijab, "klcd")}, {-1.0, ix(Gijab, "lkcd")}},
             {{1.0, ix(tau, "adkl")}}, O);
  E.contract(ix(r1, "ai"), 1.0, 1.0, {{1.0, ix(*S.FAB, "ac")}}, {{1.0, ix(t1, "ci")}}, O);
  // h_ki = F_oo(Fij, gbar, tau); FIJ = h_ki; r1 -= t1(a,k) h_ki(k,i)
  E.assign(ix(*S.FIJ, "ki"), 0.0, {f1(1.0, ix(Fij, "ki"))});
  E.contract(ix(*S.FIJ, "ki"), 1.0, 1.0, {{2.0, ix(Gijab, "klab")}, {-1.0, ix(Gijab, "lkab")}},
             {{1.0, ix(tau, "abil")}}, O);
  E.contract(ix(r1, "ai"), 1.0, -1.0, {{1.0, ix(t1, "ak")}}, {{1.0, ix(*S.FIJ, "ki")}}, O);
  // h_kc = F_ov(Fia, gbar, t1); r1 += h_kc(k,c) (2 t2(c,a,k,i) - t2(c,a,i,k) + t1(c,i) t1(a,k))
  E.assign(ix(*S.hkc, "kc"), 0.0, {f1(1.0, ix(Fia, "kc"))});
  E.contract(ix(*S.hkc, "kc"), 1.0, 1.0, {{2.0, ix(Gijab, "klcd")}, {-1.0, ix(Gijab, "lkcd")}},
             {{1.0, ix(t1, "dl")}}, O);
  // (t2(c,a,i,k) read as t2(a,c,k,i): both terms then run along i in storage)
  E.contract(ix(r1, "ai"), 1.0, 1.0, {{1.0, ix(*S.hkc, "kc")}}, {{2.0, ix(t2, "caki")}, {-1.0, ix(t2, "acki")}}, O);
  E.contract(ix(*S.tki, "ki"), 0.0, 1.0, {{1.0, ix(*S.hkc, "kc")}}, {{1.0, ix(t1, "ci")}}, O);
  E.contract(ix(r1, "ai"), 1.0, 1.0, {{1.0, ix(t1, "ak")}}, {{1.0, ix(*S.tki, "ki")}}, O);
  // r1 += (2 Gijab(k,i,c,a) - Giajb(k,a,i,c)) t1(c,k)
  E.contract(ix(r1, "ai"), 1.0, 1.0, {{2.0, ix(Gijab, "kica")}, {-1.0, ix(Giajb, "kaic")}},
             {{1.0, ix(t1, "ck")}}, O);
  // r1 += (2 Giabc(k,a,c,d) - Giabc(k,a,d,c)) tau(c,d,k,i) (:111-114) = 2 tmp2(k,a,k,i) - tmp2(k,a,i,k)
  E.custom([=](cudaStream_t st) { launch_r1_from_tmp2(o, v, tmp2, r1d, st); }, 1);
  // r1 -= (2 Gijka(l,k,i,c) - Gijka(k,l,i,c)) tau(c,a,k,l), read through
  // tau(c,a,k,l) = tau(a,c,l,k) as (2 Gijka(k,l,i,d) - Gijka(l,k,i,d)) tau(a,d,k,l):
  // the same pack of tau as F_vv's above, shared
  E.contract(ix(r1, "ai"), 1.0, -1.0, {{2.0, ix(Gijka, "klid")}, {-1.0, ix(Gijka, "lkid")}},
             {{1.0, ix(tau, "adkl")}}, O);

  // ----- R2 (ccsd_r1_r2.h:198-293) -----
  // K, P and r2u each receive their first (beta = 0) value from a ring
  // contraction and the cheaper terms accumulate after it: a tensor-core
  // product that stores C runs ~0.5 ms faster at o=32 v=320 than one that
  // reads and adds to it, while an elementwise pass pays little for the read.
  const Tensor& r2u = *S.r2u;
  const Tensor &P = *S.P, &K = *S.K;
  // j and k intermediates (:229-249) with T(d,a,i,l) = 0.5 t2(d,a,i,l) + t1(d,i) t1(a,l)
  // = tau(d,a,i,l) - 0.5 t2(d,a,i,l), packed from those two arrays where it is used
  // (not stored; two plain terms pack faster than t2 and a t1 t1 product).  j enters r2 only
  // as P(a,k,i,c) = 2 j(a,k,i,c) - k(k,a,i,c), whose ring part
  //   -2 G_cd T + (2 G_cd - G_dc) t2(a,d,i,l) + G_dc T = (2 G_cd - G_dc) (t2(a,d,i,l) - T)
  // (G_cd = Gijab(k,l,c,d), G_dc = Gijab(k,l,d,c), summed over l, d) is one
  // contraction instead of j's two and a share of k's
  const std::vector<Lin> T = {{1.0, ix(tau, "dail")}, {-0.5, ix(t2, "dail")}};
  E.contract(ix(K, "kaic"), 0.0, -1.0, {{1.0, ix(Gijab, "kldc")}}, T, R);
  E.assign(ix(K, "kaic"), 1.0, {f1(1.0, ix(Giajb, "kaic"))});
  E.contract(ix(K, "kaic"), 1.0, -1.0, {{1.0, ix(Gijka, "klic")}}, {{1.0, ix(t1, "al")}}, O);
  const double *Kd = K.d, *Pd = P.d;
  double *dK = S.diagK->d, *dP = S.diagP->d;
  E.custom([=](cudaStream_t st) { launch_diag_snapshot(o, v, 0, Kd, dK, st); }, 1);
  E.contract(ix(K, "kaic"), 1.0, 1.0, {{1.0, ix(Giabc, "kadc")}}, {{1.0, ix(t1, "di")}}, O);
  E.contract(ix(P, "akic"), 0.0, 1.0, {{2.0, ix(Gijab, "klcd")}, {-1.0, ix(Gijab, "kldc")}},
             {{1.0, ix(t2, "adil")}, {0.5, ix(t2, "dail")}, {-1.0, ix(tau, "dail")}}, R);
  // the rest of 2 j - k: 2 Gijab(i,k,a,c) - Giajb(k,a,i,c) - (2 Gijka(l,k,i,c) -
  // Gijka(k,l,i,c)) t1(a,l) + (2 Giabc(k,a,c,d) - Giabc(k,a,d,c)) t1(d,i)
  E.assign(ix(P, "akic"), 1.0, {f1(2.0, ix(Gijab, "ikac")), f1(-1.0, ix(Giajb, "kaic"))});
  E.contract(ix(P, "akic"), 1.0, -1.0, {{2.0, ix(Gijka, "lkic")}, {-1.0, ix(Gijka, "klic")}},
             {{1.0, ix(t1, "al")}}, O);
  E.custom([=](cudaStream_t st) { launch_diag_snapshot(o, v, 1, Pd, dP, st); }, 1);
  E.contract(ix(P, "akic"), 1.0, 1.0, {{2.0, ix(Giabc, "kacd")}, {-1.0, ix(Giabc, "kadc")}},
             {{1.0, ix(t1, "di")}}, O);
  // r2 += 0.5 (2 j(a,k,i,c) - k(k,a,i,c)) (2 t2(c,b,k,j) - t2(b,c,k,j))   (:251-252)
  E.contract(ix(r2u, "abij"), 0.0, 0.5, {{1.0, ix(P, "akic")}}, {{2.0, ix(t2, "cbkj")}, {-1.0, ix(t2, "bckj")}},
             R);
  // permutation part (:206-212)
  // r2u -= Y1(k,a,j,i) t1(b,k) [image of Y1(k,b,i,j) t1(a,k)] + Gijka(j,i,k,a) t1(b,k)
  //        + Y2(i,k,a,j) t1(b,k) + tmp2(k,a,j,i) t1(b,k) [the ladder's t1 terms, :278-280]
  E.contract(ix(r2u, "abij"), 1.0, 1.0, {{1.0, ix(Giabc, "icab")}}, {{1.0, ix(t1, "cj")}}, O);
  E.contract(ix(*S.Y1, "kbij"), 0.0, 1.0, {{1.0, ix(Giajb, "kbic")}}, {{1.0, ix(t1, "cj")}}, O);
  E.contract(ix(*S.Y2, "ikaj"), 0.0, 1.0, {{1.0, ix(Gijab, "ikac")}}, {{1.0, ix(t1, "cj")}}, O);
  E.contract(ix(r2u, "abij"), 1.0, -1.0,
             {{1.0, ix(*S.Y1, "kaji")}, {1.0, ix(Gijka, "jika")}, {1.0, ix(*S.Y2, "ikaj")}, {1.0, ix(*S.tmp2, "kaji")}},
             {{1.0, ix(t1, "bk")}}, O);
  // g_ki = F_OO(FIJ, Fia, gbar_ijka, t1), gbar_ijka(k,l,i,c) = 2 Gijka(k,l,i,c) - Gijka(l,k,i,c)
  E.assign(ix(*S.gki, "ki"), 0.0, {f1(1.0, ix(*S.FIJ, "ki"))});
  E.contract(ix(*S.gki, "ki"), 1.0, 1.0, {{1.0, ix(Fia, "kc")}}, {{1.0, ix(t1, "ci")}}, O);
  E.contract(ix(*S.gki, "ki"), 1.0, 1.0, {{2.0, ix(Gijka, "klic")}, {-1.0, ix(Gijka, "lkic")}},
             {{1.0, ix(t1, "cl")}}, O);
  // g_ac = F_VV(FAB, Fia, gbar_iabc, t1), gbar_iabc(k,a,d,c) = 2 Giabc(k,a,d,c) - Giabc(k,a,c,d)
  // (the reference's 4-argument F_VV adds + Fia(k,c) t1(a,k); kept as written)
  E.assign(ix(*S.gac, "ac"), 0.0, {f1(1.0, ix(*S.FAB, "ac"))});
  E.contract(ix(*S.gac, "ac"), 1.0, 1.0, {{1.0, ix(Fia, "kc")}}, {{1.0, ix(t1, "ak")}}, O);
  // the gbar_iabc t1 term from the diagonals i = k of the Giabc t1 terms of K and P
  // (kernels.cu): no pass over Giabc of its own
  double* gacd = S.gac->d;
  E.custom([=](cudaStream_t st) { launch_gac_from_diagonals(o, v, Kd, Pd, dK, dP, gacd, st); }, 1);
  // r2 += g_ac(a,c) t2(c,b,i,j) - g_ki(k,i) t2(a,b,k,j)
  E.contract(ix(r2u, "abij"), 1.0, 1.0, {{1.0, ix(*S.gac, "ac")}}, {{1.0, ix(t2, "cbij")}}, O);
  E.contract(ix(r2u, "abij"), 1.0, -1.0, {{1.0, ix(*S.gki, "ki")}}, {{1.0, ix(t2, "abkj")}}, O);
  // tmp(a,b,i,j) = k(k,a,i,c) t2(c,b,j,k); r2 -= 0.5 tmp(a,b,i,j) + tmp(b,a,i,j)   (:254-256)
  // (t2(c,b,j,k) read as t2(b,c,k,j): its rows (b,j) then run along j in storage)
  E.contract(ix(*S.tmp, "abij"), 0.0, 1.0, {{1.0, ix(K, "kaic")}}, {{1.0, ix(t2, "bckj")}}, R);
  // r2(a,b,i,j) = r2u(a,b,i,j) + r2u(b,a,j,i) + Gijab(i,j,a,b)   (:260-262), with the
  // tmp terms, is added by the assembly pass below (g_abij(a,b,i,j) = Gijab(i,j,a,b),
  // stored in r2's order)
  const double *r2u_d = r2u.d, *tmp_d = S.tmp->d, *gab_d = S.g_abij->d;
  // hole-hole ladder: W_oooo (intermediates :182-193), r2 += W(k,l,i,j) tau(a,b,k,l)
  const Tensor& W = *S.W;
  E.assign(ix(W, "klij"), 0.0, {f1(1.0, ix(Gijkl, "klij"))});
  E.contract(ix(W, "klij"), 1.0, 1.0, {{1.0, ix(Gijka, "klic")}}, {{1.0, ix(t1, "cj")}}, O);
  E.contract(ix(W, "klij"), 1.0, 1.0, {{1.0, ix(Gijka, "lkjc")}}, {{1.0, ix(t1, "ci")}}, O);
  if (direct) {
    E.contract(ix(W, "klij"), 1.0, 1.0, {{1.0, ix(Gijab, "klcd")}}, {{1.0, ix(tau, "cdij")}}, O);
    E.contract(ix(r2, "abij"), 0.0, 1.0, {{1.0, ix(W, "klij")}}, {{1.0, ix(tau, "abkl")}}, O);
    E.custom([=](cudaStream_t st) { launch_r2_assemble(o, v, r2u_d, tmp_d, gab_d, nullptr, nullptr, true, r2d, st); },
             1);
    // integral-direct (:282-286): r2 += Ca(p,a) u(p,r,i,j) Ca(r,b); the T1 parts
    // (Ci u terms) are the tmp2 terms of r2u above
    E.contract(ix(*S.U1, "arij"), 0.0, 1.0, {{1.0, ix(*S.Ca, "pa")}}, {{1.0, ix(*S.u, "prij")}}, O);
    E.contract(ix(r2, "abij"), 1.0, 1.0, {{1.0, ix(*S.U1, "arij")}}, {{1.0, ix(*S.Ca, "rb")}}, O);
    return;
  }
  // otherwise as pair products (kernels.cu): W+- from the Gijkl and Gijka t1
  // parts of W, plus Gijab's pair factors times tau+-; their products with
  // tau+- add to the particle-particle ladder's B+- below
  {
    const double* Wd = W.d;
    double *Wt = S.Wt->d, *Wm = minus ? S.Wm->d : nullptr;
    E.custom([=](cudaStream_t st) { launch_pair_combine_oo(o, Wd, Wt, Wm, st); }, 1);
    E.contract(ix(*S.Wt, "PS"), 1.0, 1.0, {{1.0, ix(*S.Gtp, "PQ")}}, {{1.0, ix(*S.taup, "QS")}}, O);
    if (minus) E.contract(ix(*S.Wm, "XZ"), 1.0, 1.0, {{1.0, ix(*S.Gtm, "XY")}}, {{1.0, ix(*S.taum, "YZ")}}, O);
  }
  // particle-particle ladder (:275, :289): r2 += tau(c,d,i,j) Gabcd(a,b,c,d) as sums
  // over c <= d of the pair-(anti)symmetric combinations (taup / taum from above)
  double *Bp = S.Bp->d, *Bm = S.Bm->d;
  if (S.naux == 0) {
    E.contract(ix(*S.Bp, "PS"), 0.0, 1.0, {{1.0, ix(*S.Gp, "PQ")}}, {{1.0, ix(*S.taup, "QS")}}, L);
    if (minus) E.contract(ix(*S.Bm, "XZ"), 0.0, 1.0, {{1.0, ix(*S.Gm, "XY")}}, {{1.0, ix(*S.taum, "YZ")}}, L);
  } else {
    // density fitting, lazy (ab|cd) (the reference's direct-DF ladder,
    // ccsd_r1_r2.h:497-508): per block of a, <ab|cd> = sum_K (K|ac)(K|bd) on
    // the tensor cores, its G+- rows, and those rows of the pair products
    for (const auto& bp : S.df_blocks) {
      const CcsdTensors::DfBlock& B = *bp;
      E.contract(ix(B.g, "abcd"), 0.0, 1.0, {{1.0, ix(B.xa, "acK")}}, {{1.0, ix(B.xb, "bdK")}}, L);
      const int64_t a0 = B.a0, a1 = B.a1;
      const double* gd = B.g.d;
      double *gp = B.gp.d, *gm = B.gm.d;
      E.custom([=](cudaStream_t st) { launch_build_gpm_rows(a0, a1, v, gd, gp, gm, st); }, 1);
      E.contract(ix(B.bp, "PS"), 0.0, 1.0, {{1.0, ix(B.gp, "PQ")}}, {{1.0, ix(*S.taup, "QS")}}, L);
      if (minus && B.rows_m > 0)
        E.contract(ix(B.bm, "XZ"), 0.0, 1.0, {{1.0, ix(B.gm, "XY")}}, {{1.0, ix(*S.taum, "YZ")}}, L);
    }
  }
  E.contract(ix(*S.Bp, "RS"), 1.0, 1.0, {{1.0, ix(*S.taup, "RP")}}, {{1.0, ix(*S.Wt, "PS")}}, O);
  if (minus) E.contract(ix(*S.Bm, "UZ"), 1.0, 1.0, {{1.0, ix(*S.taum, "UX")}}, {{1.0, ix(*S.Wm, "XZ")}}, O);
  // r2 = the symmetrised r2u and tmp terms, g_abij and both ladders' pair products
  E.custom(
      [=](cudaStream_t st) { launch_r2_assemble(o, v, r2u_d, tmp_d, gab_d, Bp, minus ? Bm : nullptr, false, r2d, st); },
      1);
}

}  // namespace gbcc

extern "C" int gbcc_testing_df_block_rows(int64_t rows) {
  if (rows < 0) return GBCC_ERR_INVALID_ARG;
  gbcc::g_df_block_rows = rows;
  return GBCC_OK;
}
