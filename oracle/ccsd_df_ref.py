"""FP64 CPU oracle for the density-fitted closed-shell CCSD residual.

TEST INFRASTRUCTURE ONLY, like ``oracle/ccsd_ref.py``: only ``tests/`` may
import it.  The product path never does.

It restates MPQC's density-fitted residual with the lazy (direct) ladder: the
(ab|cd) block is never stored, and the T1 parts of the ladder are folded into
a modified three-index factor.  The restatement follows the reference line by
line (paths relative to the MPQC source tree):

  src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:136-184  compute_cs_ccsd_r1_df
  src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:309-520  compute_cs_ccsd_r2_df, the
      branch with neither Gabcd nor factor matrices (:497-508)
  src/mpqc/chemistry/qc/lcao/integrals/integral_builder.h:228-300
      DirectDFIntegralBuilder: in physical notation <pq|rs> = sum_K bra(K,p,r) ket(K,q,s)

Three-index factors, in MPQC's annotation order:

    Xai[K,a,i] = (K|ai)    Xab[K,a,b] = (K|ab)    Xij[K,i,j] = (K|ij)

with (pq|rs) = sum_K X(K,p,q) X(K,r,s).  The remaining four-index blocks the
reference still reads (Gijab, Gijkl, Giajb, Gijka) come in ``Integrals`` as for
the standard residual; Giabc and Gabcd are not used.

Pinned without running the reference: with all blocks built from the same
factors, this residual must equal the standard one (``oracle/ccsd_ref.py``) to
rounding (``tests/test_oracle_df.py``).
"""
from __future__ import annotations

import numpy as np

from .ccsd_ref import F_OO, W_oooo, Integrals, _es, make_tau


def compute_cs_ccsd_r1_df(t1, t2, tau, ints: Integrals, Xai, Xab, Xij):
    """ccsd_r1_r2.h:136-184.  Writes ints.FAB / ints.FIJ like the standard R1."""
    # X_ai_tau(X,a,i) = 2 Xai(X,b,j) tau(a,b,i,j) - Xai(X,b,j) tau(a,b,j,i)      :148-149
    X_ai_tau = 2.0 * _es("Xbj,abij->Xai", Xai, tau) - _es("Xbj,abji->Xai", Xai, tau)
    r1 = ints.Fia.T - 2.0 * _es("ki,ak->ai", _es("kc,ci->ki", ints.Fia, t1), t1)       # :153
    h_ac = ints.Fab - _es("Kal,Kcl->ac", X_ai_tau, Xai)                                # :156
    ints.FAB = h_ac
    r1 = r1 + _es("ac,ci->ai", h_ac, t1)                                               # :158
    h_ki = ints.Fij + _es("Kci,Kck->ki", X_ai_tau, Xai)                                # :162
    ints.FIJ = h_ki
    r1 = r1 - _es("ak,ki->ai", t1, h_ki)                                               # :164
    h_kc = ints.Fia + _es("klcd,dl->kc", 2.0 * ints.Gijab - _es("kldc->klcd", ints.Gijab), t1)  # :168-170
    x = 2.0 * t2 - _es("caik->caki", t2) + _es("ci,ak->caki", t1, t1)
    r1 = r1 + _es("kc,caki->ai", h_kc, x)                                              # :171-172
    y = 2.0 * ints.Gijab - _es("kaic->kica", ints.Giajb)
    r1 = r1 + _es("kica,ck->ai", y, t1)                                                # :175-176
    r1 = r1 + _es("Kci,Kac->ai", X_ai_tau, Xab)                                        # :178
    r1 = r1 - _es("Kal,Kli->ai", X_ai_tau, Xij)                                        # :180
    return r1


def compute_cs_ccsd_r2_df(t1, t2, tau, ints: Integrals, Xai, Xab, Xij):
    """ccsd_r1_r2.h:309-520 with the lazy density-fitted ladder (:497-508).
    Needs ints.FIJ / FAB from compute_cs_ccsd_r1_df."""
    # permutation part, :317-324
    X_ab_t1 = _es("Kab,bi->Kai", Xab, t1)
    r2 = (_es("Kbj,Kai->abij", X_ab_t1, Xai)
          - _es("Kbj,Kki,ak->abij", X_ab_t1, Xij, t1))
    y = ints.Gijka + _es("ikac,cj->jika", ints.Gijab, t1)
    r2 = r2 - _es("jika,bk->abij", y, t1)
    # g intermediates, :326-340
    g_ijka_bar = 2.0 * ints.Gijka - _es("jika->ijka", ints.Gijka)
    g_ki = F_OO(ints.FIJ, ints.Fia, g_ijka_bar, t1)
    g_ac = (ints.FAB - _es("kc,ak->ac", ints.Fia, t1)
            + 2.0 * _es("Kdk,dk,Kac->ac", Xai, t1, Xab)
            - _es("Kak,Kck->ac", X_ab_t1, Xai))
    r2 = r2 + _es("ac,cbij->abij", g_ac, t2) - _es("ki,abkj->abij", g_ki, t2)
    # j and k intermediates, :342-358
    T = 0.5 * t2 + _es("di,bl->dbil", t1, t1)
    j_akic = (_es("ikac->akic", ints.Gijab)
              - _es("lkic,al->akic", ints.Gijka, t1)
              + _es("Kai,Kck->akic", X_ab_t1, Xai)
              - _es("xdl,dail,xck->akic", Xai, T, Xai)
              + 0.5 * _es("klcd,adil->akic", 2.0 * ints.Gijab - _es("kldc->klcd", ints.Gijab), t2))
    k_kaic = (ints.Giajb
              - _es("klic,al->kaic", ints.Gijka, t1)
              + _es("Kdk,di,Kac->kaic", Xai, t1, Xab)
              - _es("kldc,dail->kaic", ints.Gijab, T))
    # ring apply, :360-365
    u = 2.0 * j_akic - _es("kaic->akic", k_kaic)
    w = 2.0 * t2 - _es("bckj->cbkj", t2)
    r2 = r2 + 0.5 * _es("akic,cbkj->abij", u, w)
    tmp = _es("kaic,cbjk->abij", k_kaic, t2)
    r2 = r2 - (0.5 * tmp + _es("baij->abij", tmp))
    # symmetrise and add Gijab(i,j,a,b), :368-369
    r2 = r2 + _es("baji->abij", r2)
    r2 = r2 + _es("ijab->abij", ints.Gijab)
    # hole-hole ladder, :371-377
    a_klij = W_oooo(ints.Gijkl, ints.Gijka, ints.Gijab, tau, t1)
    r2 = r2 + _es("klij,abkl->abij", a_klij, tau)
    # lazy particle-particle ladder, :497-508:
    #   X(K,a,b) = 0.5 Xab(K,a,b) - Xai(K,b,i) t1(a,i)
    #   g(a,b,c,d) = sum_K Xab(K,a,c) X(K,b,d)   (physical notation)
    #   b(a,b,i,j) = tau(c,d,i,j) g(a,b,c,d);  b += b(b,a,j,i)
    X_ab_mod = 0.5 * Xab - _es("Kbi,ai->Kab", Xai, t1)
    g_abcd = _es("Kac,Kbd->abcd", Xab, X_ab_mod)
    b_abij = _es("cdij,abcd->abij", tau, g_abcd)
    b_abij = b_abij + _es("baji->abij", b_abij)
    return r2 + b_abij


def residual_df(t1, t2, ints: Integrals, Xai, Xab, Xij):
    """One density-fitted R1 then R2 evaluation (R1 sets ints.FIJ / FAB)."""
    tau = make_tau(t1, t2)
    r1 = compute_cs_ccsd_r1_df(t1, t2, tau, ints, Xai, Xab, Xij)
    r2 = compute_cs_ccsd_r2_df(t1, t2, tau, ints, Xai, Xab, Xij)
    return r1, r2


def df_factors(B, o):
    """(Xai, Xab, Xij) from a factor B[K,p,q] over the full space (occupied
    first) with (pq|rs) = sum_K B[K,p,q] B[K,r,s]."""
    return (np.ascontiguousarray(B[:, o:, :o]), np.ascontiguousarray(B[:, o:, o:]),
            np.ascontiguousarray(B[:, :o, :o]))
