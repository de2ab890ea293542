"""FP64 CPU oracle for the closed-shell CCSD amplitude solver.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference legs may
import it.  The product path (``mpqc_gb300`` and ``libgbcc``) never does.

It restates, in numpy FP64, the spin-adapted closed-shell CCSD equations of
MPQC (ValeevGroup/mpqc), one einstein-index expression of the reference per
line.  Every tensor is stored in the index order of its MPQC annotation:

    Fia[i,a]  Fij[i,j]  Fab[a,b]              (Fock blocks, ``cc::Integrals``)
    Gijab[i,j,a,b] = <ij|ab>   Gijkl[i,j,k,l] = <ij|kl>
    Giajb[i,a,j,b] = <ia|jb>   Gijka[i,j,k,a] = <ij|ka>
    Giabc[i,a,b,c] = <ia|bc>   Gabcd[a,b,c,d] = <ab|cd>
    t1[a,i]   t2[a,b,i,j]   tau[a,b,i,j]

so that an MPQC expression such as ``Giabc("k,a,d,c") * t1("d,i")`` reads as
``einsum('kadc,di->...', Giabc, t1)``.

Sources restated (paths relative to the MPQC source tree):
  src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:70-124   compute_cs_ccsd_r1 (standard)
  src/mpqc/chemistry/qc/lcao/cc/ccsd_r1_r2.h:198-293  compute_cs_ccsd_r2 (standard)
  src/mpqc/chemistry/qc/lcao/cc/ccsd_intermediates.h:57-193  F_oo F_vv F_ov F_OO F_VV W_oooo
  src/mpqc/chemistry/qc/lcao/cc/solvers.h:165-258     jacobi_update_t2_abij / _t1_ai
  src/mpqc/chemistry/qc/lcao/cc/solvers.h:1152-1158   JacobiDIISSolver::update_only
  src/mpqc/chemistry/qc/cc/solvers.h:60-63,112-121,141-152  error, DIIS update, convergence
  src/mpqc/chemistry/qc/lcao/cc/ccsd.h:331-477        CCSD::compute_ccsd loop and energy

The DIIS extrapolation lives in TiledArray (``TA::DIIS``, not part of the MPQC
tree).  ``PulayDIIS`` below restates Pulay's method (Chem. Phys. Lett. 73, 393
(1980)) with MPQC's parameters (diis_start=1, n_diis=8, diis_damp=0,
diis_ngroup=1, diis_group_nstart=1; cc/solvers.h:93-95).  Its subspace solve is
Gaussian elimination with partial pivoting on the bordered B matrix normalised
by its oldest kept diagonal entry, dropping the oldest vector while |det| of
that matrix is below DIIS_DET_MIN; the GPU solver performs the identical
arithmetic.  This rule is pinned by the iteration trace the reference recorded
for water/6-31G (its validation output h2o-ccsd-direct-631g.out:291-303, a
build that started from MP2 amplitudes): ``solve_ccsd(..., initial="mp2")``
reproduces all 13 recorded (dE, error, E) rows to their printed digits.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def _es(spec, *ops):
    return np.einsum(spec, *ops, optimize=True)


# ---------------------------------------------------------------------------
# intermediates: ccsd_intermediates.h
# ---------------------------------------------------------------------------

def F_oo(f_oo, g_ijab_bar, tau):
    """ccsd_intermediates.h:57-63: F_oo(k,i) = f_oo(k,i) + gbar(k,l,a,b) tau(a,b,i,l)."""
    return f_oo + _es("klab,abil->ki", g_ijab_bar, tau)


def F_vv(f_vv, g_ijab_bar, tau):
    """ccsd_intermediates.h:71-77: F_vv(a,c) = f_vv(a,c) - gbar(k,l,c,d) tau(a,d,k,l)."""
    return f_vv - _es("klcd,adkl->ac", g_ijab_bar, tau)


def F_ov(f_ov, g_ijab_bar, t1):
    """ccsd_intermediates.h:89-95: F_ov(k,c) = f_ov(k,c) + gbar(k,l,c,d) t1(d,l)."""
    return f_ov + _es("klcd,dl->kc", g_ijab_bar, t1)


def F_OO(F_oo_, f_ov, g_ijka_bar, t1):
    """ccsd_intermediates.h:105-112 (4-argument form used by R2)."""
    return F_oo_ + _es("kc,ci->ki", f_ov, t1) + _es("klic,cl->ki", g_ijka_bar, t1)


def F_VV(F_vv_, f_ov, g_iabc_bar, t1):
    """ccsd_intermediates.h:141-148 (4-argument form used by R2).

    Mirrors the reference as written, including the ``+ f_ov(k,c) t1(a,k)`` sign
    (the term vanishes for canonical orbitals, where f_ov = 0)."""
    return F_vv_ + _es("kc,ak->ac", f_ov, t1) + _es("kadc,dk->ac", g_iabc_bar, t1)


def W_oooo(g_ijkl, g_ijka, g_ijab, tau, t1):
    """ccsd_intermediates.h:182-193."""
    return (g_ijkl + _es("klic,cj->klij", g_ijka, t1) + _es("lkjc,ci->klij", g_ijka, t1)
            + _es("klcd,cdij->klij", g_ijab, tau))


# ---------------------------------------------------------------------------
# residuals: ccsd_r1_r2.h
# ---------------------------------------------------------------------------

@dataclass
class Integrals:
    """cc::Integrals (ccsd_r1_r2.h:24-56), standard-method members only."""
    Fia: np.ndarray
    Fij: np.ndarray
    Fab: np.ndarray
    Gijab: np.ndarray
    Gijkl: np.ndarray
    Giajb: np.ndarray
    Gijka: np.ndarray
    Giabc: np.ndarray
    Gabcd: np.ndarray
    FIJ: np.ndarray | None = None
    FAB: np.ndarray | None = None
    # the integral-direct members (method "direct"): MO coefficients of the
    # active occupied and the virtual orbitals, Ci[p,k] and Ca[p,a]
    Ci: np.ndarray | None = None
    Ca: np.ndarray | None = None

    @property
    def o(self):
        return self.Fij.shape[0]

    @property
    def v(self):
        return self.Fab.shape[0]


def make_tau(t1, t2):
    """ccsd.h:342,389: tau(a,b,i,j) = t2(a,b,i,j) + t1(a,i) t1(b,j)."""
    return t2 + _es("ai,bj->abij", t1, t1)


def compute_u2_u11(t1, t2, ints: Integrals, G_ao):
    """ccsd.h:580-603: U(p,r,i,j) = (t2(a,b,i,j) Ca(q,a) Ca(s,b) + tc(i,q) tc(j,s)) (p q|r s)
    with tc(i,q) = Ca(q,c) t1(c,i) and G_ao[p,q,r,s] = (pq|rs) over atomic orbitals."""
    tc = _es("qc,ci->iq", ints.Ca, t1)
    tau_ao = _es("abij,qa,sb->qsij", t2, ints.Ca, ints.Ca) + _es("iq,js->qsij", tc, tc)
    return _es("pqrs,qsij->prij", G_ao, tau_ao)


def compute_cs_ccsd_r1(t1, t2, tau, ints: Integrals, u=None):
    """ccsd_r1_r2.h:70-124 (standard method; with u the integral-direct branch
    of :116-118).  Writes ints.FAB / ints.FIJ."""
    r1 = ints.Fia.T - 2.0 * _es("ki,ak->ai", _es("kc,ci->ki", ints.Fia, t1), t1)      # :82-83
    g_ijab_bar = 2.0 * ints.Gijab - _es("jiab->ijab", ints.Gijab)                     # :86
    h_ac = F_vv(ints.Fab, g_ijab_bar, tau)                                            # :88
    ints.FAB = h_ac
    r1 = r1 + _es("ac,ci->ai", h_ac, t1)                                              # :90
    h_ki = F_oo(ints.Fij, g_ijab_bar, tau)                                            # :94
    ints.FIJ = h_ki
    r1 = r1 - _es("ak,ki->ai", t1, h_ki)                                              # :96
    h_kc = F_ov(ints.Fia, g_ijab_bar, t1)                                             # :100
    x = 2.0 * t2 - _es("caik->caki", t2) + _es("ci,ak->caki", t1, t1)          # 2 t2(c,a,k,i) - t2(c,a,i,k) + t1(c,i) t1(a,k)
    r1 = r1 + _es("kc,caki->ai", h_kc, x)                                             # :102-103
    y = 2.0 * ints.Gijab - _es("kaic->kica", ints.Giajb)
    # 2 Gijab(k,i,c,a) - Giajb(k,a,i,c), laid out (k,i,c,a)
    r1 = r1 + _es("kica,ck->ai", y, t1)                                               # :106-107
    if u is None:
        g_iabc_bar = 2.0 * ints.Giabc - _es("kadc->kacd", ints.Giabc)                 # :111-112
        r1 = r1 + _es("kacd,cdki->ai", g_iabc_bar, tau)                               # :113
    else:
        r1 = r1 + _es("prki,pk,ra->ai", 2.0 * u - _es("prik->prki", u), ints.Ci, ints.Ca)  # :116-118
    g_lkic = 2.0 * ints.Gijka - _es("klic->lkic", ints.Gijka)  # 2 Gijka(l,k,i,c) - Gijka(k,l,i,c)
    r1 = r1 - _es("lkic,cakl->ai", g_lkic, tau)                                       # :120-121
    return r1


def compute_cs_ccsd_r2(t1, t2, tau, ints: Integrals, u=None):
    """ccsd_r1_r2.h:198-293 (standard method; with u the integral-direct ladder
    of :282-286).  Needs ints.FIJ/FAB from R1."""
    # permutation part, :206-212
    x = ints.Giabc - _es("kbic,ak->icab", ints.Giajb, t1)   # Giabc(i,c,a,b) - Giajb(k,b,i,c) t1(a,k)
    r2 = _es("icab,cj->abij", x, t1)
    y = ints.Gijka + _es("ikac,cj->jika", ints.Gijab, t1)
    # Gijka(j,i,k,a) + Gijab(i,k,a,c) t1(c,j), laid out (j,i,k,a)
    r2 = r2 - _es("jika,bk->abij", y, t1)
    # g intermediates, :214-227
    g_ijka_bar = 2.0 * ints.Gijka - _es("jika->ijka", ints.Gijka)
    g_ki = F_OO(ints.FIJ, ints.Fia, g_ijka_bar, t1)
    g_iabc_bar = 2.0 * ints.Giabc - _es("kabd->kadb", ints.Giabc)
    g_ac = F_VV(ints.FAB, ints.Fia, g_iabc_bar, t1)
    r2 = r2 + _es("ac,cbij->abij", g_ac, t2) - _es("ki,abkj->abij", g_ki, t2)
    # j and k intermediates, :229-249
    T = 0.5 * t2 + _es("di,bl->dbil", t1, t1)
    j_akic = (_es("ikac->akic", ints.Gijab)
              - _es("lkic,al->akic", ints.Gijka, t1)
              + _es("kacd,di->akic", ints.Giabc, t1)
              - _es("klcd,dail->akic", ints.Gijab, T)
              + 0.5 * _es("klcd,adil->akic",
                          2.0 * ints.Gijab - _es("kldc->klcd", ints.Gijab), t2))
    k_kaic = (ints.Giajb
              - _es("klic,al->kaic", ints.Gijka, t1)
              + _es("kadc,di->kaic", ints.Giabc, t1)
              - _es("kldc,dail->kaic", ints.Gijab, T))
    # ring apply, :251-256
    jk = 2.0 * j_akic - _es("kaic->akic", k_kaic)
    w = 2.0 * t2 - _es("bckj->cbkj", t2)                 # 2 t2(c,b,k,j) - t2(b,c,k,j)
    r2 = r2 + 0.5 * _es("akic,cbkj->abij", jk, w)
    tmp = _es("kaic,cbjk->abij", k_kaic, t2)
    r2 = r2 - (0.5 * tmp + _es("baij->abij", tmp))
    # symmetrise and add Gijab(i,j,a,b), :259-262
    r2 = r2 + _es("baji->abij", r2)
    r2 = r2 + _es("ijab->abij", ints.Gijab)
    # hole-hole ladder, :264-270
    a_klij = W_oooo(ints.Gijkl, ints.Gijka, ints.Gijab, tau, t1)
    r2 = r2 + _es("klij,abkl->abij", a_klij, tau)
    # particle-particle ladder, :272-280
    if u is not None:                                                                 # :282-286
        b_abij = (_es("prij,rb,pa->abij", u, ints.Ca, ints.Ca)
                  - _es("rk,bk,prij,pa->abij", ints.Ci, t1, u, ints.Ca)
                  - _es("prij,pk,rb,ak->abij", u, ints.Ci, ints.Ca, t1))
        return r2 + b_abij
    b_abij = _es("cdij,abcd->abij", tau, ints.Gabcd)
    tmp2 = _es("kacd,cdij->kaij", ints.Giabc, tau)
    b_abij = b_abij - _es("kaji,bk->abij", tmp2, t1)
    b_abij = b_abij - _es("kbij,ak->abij", tmp2, t1)
    return r2 + b_abij


def residual(t1, t2, ints: Integrals, G_ao=None):
    """One R1 then R2 evaluation (R1 first: it sets ints.FIJ/FAB read by R2).
    With AO integrals G_ao (and ints.Ca / Ci) the integral-direct branches
    (ccsd.h:581-603 U, ccsd_r1_r2.h:116-118, 282-286), as method "direct"."""
    tau = make_tau(t1, t2)
    u = compute_u2_u11(t1, t2, ints, G_ao) if G_ao is not None else None
    r1 = compute_cs_ccsd_r1(t1, t2, tau, ints, u)
    r2 = compute_cs_ccsd_r2(t1, t2, tau, ints, u)
    return r1, r2


# ---------------------------------------------------------------------------
# solver: Jacobi + DIIS, error and convergence
# ---------------------------------------------------------------------------

def jacobi_update_t1_ai(r1, eps_o, eps_v):
    """lcao/cc/solvers.h:223-258: delta(a,i) = r1(a,i) / (e_i - e_a)."""
    return r1 / (eps_o[None, :] - eps_v[:, None])


def jacobi_update_t2_abij(r2, eps_o, eps_v):
    """lcao/cc/solvers.h:165-210: delta(a,b,i,j) = r2 / (e_i + e_j - e_a - e_b)."""
    d = (eps_o[None, None, :, None] + eps_o[None, None, None, :]
         - eps_v[:, None, None, None] - eps_v[None, :, None, None])
    return r2 / d


def solver_error(r1, r2):
    """cc/solvers.h:60-63: sqrt(|r1|^2 + |r2|^2) / (size(r1) + size(r2))."""
    return math.sqrt(float(np.vdot(r1, r1) + np.vdot(r2, r2))) / (r1.size + r2.size)


def is_converged(target_precision, error, dE):
    """cc/solvers.h:141-152 (precision_margin_energy = 0.1)."""
    return dE <= target_precision * 0.1 and error <= target_precision


# |det| below which the bordered DIIS matrix counts as singular and the oldest
# stored vector is dropped.  TiledArray's TA::DIIS makes the same test on the
# matrix normalised by the oldest kept B entry; the water 6-31G iteration trace
# the reference recorded (tests/validation/reference/outputs/
# h2o-ccsd-direct-631g.out:291-303) fixes the threshold between 8.7e-16 and
# 4.1e-15 (the decisive determinants of that run are 1.52e-14 kept, 8.72e-16
# dropped, 4.06e-15 kept).
DIIS_DET_MIN = 1.0e-15


def gepp_solve(A, rhs):
    """Gaussian elimination with partial pivoting.  Returns ``(x, |det A|)``,
    ``|det A|`` being the product of the pivots (``x`` is None when a pivot is
    exactly zero).  The GPU subspace solve runs exactly these operations in the
    same order."""
    A = np.array(A, dtype=np.float64, copy=True)
    b = np.array(rhs, dtype=np.float64, copy=True)
    n = A.shape[0]
    det = 1.0
    for col in range(n):
        p = col + int(np.argmax(np.abs(A[col:, col])))
        if A[p, col] == 0.0:
            return None, 0.0
        det *= abs(A[p, col])
        if p != col:
            A[[col, p]] = A[[p, col]]
            b[[col, p]] = b[[p, col]]
        for r in range(col + 1, n):
            f = A[r, col] / A[col, col]
            A[r, col:] -= f * A[col, col:]
            b[r] -= f * b[col]
    x = np.zeros(n)
    for r in range(n - 1, -1, -1):
        s = b[r]
        for c in range(r + 1, n):
            s -= A[r, c] * x[c]
        x[r] = s / A[r, r]
    return x, det


@dataclass
class PulayDIIS:
    """Pulay DIIS over {t1,t2} with residual {r1,r2} (see module docstring)."""
    start: int = 1
    ndiis: int = 8
    damping: float = 0.0
    ngroup: int = 1
    ngroupdiis: int = 1
    iter: int = 0
    xs: list = field(default_factory=list)
    es: list = field(default_factory=list)
    B: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    last_coeffs: np.ndarray | None = None
    last_nskip: int = 0

    @staticmethod
    def dot(e1, e2):
        return float(sum(np.vdot(a, b) for a, b in zip(e1, e2)))

    def extrapolate(self, x, e):
        self.iter += 1
        if len(self.es) == self.ndiis:
            self.xs.pop(0)
            self.es.pop(0)
            self.B = self.B[1:, 1:]
        self.xs.append([a.copy() for a in x])
        self.es.append([a.copy() for a in e])
        n = len(self.es)
        B = np.zeros((n, n))
        B[: n - 1, : n - 1] = self.B
        for i in range(n):
            B[i, n - 1] = B[n - 1, i] = self.dot(self.es[i], self.es[n - 1])
        self.B = B
        if self.iter < self.start:
            return x
        if self.ngroup > 1 and (self.iter - self.start) % self.ngroup >= self.ngroupdiis:
            return x
        c, nskip = self.coefficients()
        self.last_coeffs, self.last_nskip = c, nskip
        out = [np.zeros_like(a) for a in x]
        for kk, k in enumerate(range(nskip, n)):
            for o_, xk in zip(out, self.xs[k]):
                o_ += c[kk] * xk
        return out

    def coefficients(self):
        """Pulay coefficients over the newest n - nskip vectors: the bordered
        system [[0, -1], [-1, B/|B_ss|]] (s = oldest kept vector, damping on the
        diagonal) is solved for the smallest nskip whose |det| is at least
        DIIS_DET_MIN; with one vector left the coefficient is 1."""
        n = len(self.es)
        B = self.B
        for nskip in range(n):
            m = n - nskip
            b0 = abs(B[nskip, nskip])
            norm = 1.0 / b0 if b0 > 0.0 else 1.0
            A = np.zeros((m + 1, m + 1))
            A[0, 1:] = -1.0
            A[1:, 0] = -1.0
            A[1:, 1:] = B[nskip:, nskip:] * norm
            for i in range(1, m + 1):
                A[i, i] *= 1.0 + self.damping
            rhs = np.zeros(m + 1)
            rhs[0] = -1.0
            sol, det = gepp_solve(A, rhs)
            if sol is not None and (det >= DIIS_DET_MIN or nskip == n - 1):
                return sol[1:], nskip
        return np.array([1.0]), n - 1


@dataclass
class SolveResult:
    e_corr: float
    t1: np.ndarray
    t2: np.ndarray
    iters: int
    converged: bool
    history: list


def solve_ccsd(ints: Integrals, eps_o, eps_v, target_precision=1e-9, max_iter=30,
               diis_start=1, n_diis=8, diis_damp=0.0, diis_ngroup=1, diis_group_nstart=1,
               initial="zero"):
    """ccsd.h:331-477: t=0 start, residual-augmented energy, Jacobi+DIIS loop.

    ``initial="mp2"`` starts instead from t1 = 0, t2 = g_abij / D_abij with the
    MP2 energy as the previous energy, as MPQC builds of 2017 did (the loop is
    otherwise the same; ``history[k]`` is then row k of their iteration table)."""
    o, v = ints.o, ints.v
    f_ai = ints.Fia.T.copy()
    g_abij = ints.Gijab.transpose(2, 3, 0, 1).copy()
    t1 = np.zeros((v, o))
    t2 = np.zeros((v, v, o, o))
    E1 = 0.0
    if initial == "mp2":
        D2 = (eps_o[None, None, :, None] + eps_o[None, None, None, :]
              - eps_v[:, None, None, None] - eps_v[None, :, None, None])
        t2 = g_abij / D2
        E1 = ccsd_energy(ints, t1, t2)
    elif initial != "zero":
        raise ValueError(f"initial guess {initial!r}")
    tau = make_tau(t1, t2)
    if initial == "zero":
        r1, r2 = f_ai.copy(), g_abij.copy()
    else:
        r1 = compute_cs_ccsd_r1(t1, t2, tau, ints)
        r2 = compute_cs_ccsd_r2(t1, t2, tau, ints)
    diis = PulayDIIS(diis_start, n_diis, diis_damp, diis_ngroup, diis_group_nstart)
    it = 0
    converged = False
    history = []
    while it < max_iter:
        error = solver_error(r1, r2)
        E0 = E1
        E1 = (2.0 * float(np.vdot(f_ai + r1, t1))
              + float(np.vdot(g_abij + r2, 2.0 * tau - tau.transpose(1, 0, 2, 3))))
        dE = abs(E0 - E1)
        history.append((it, dE, error, E1))
        if it == 0 or not is_converged(target_precision, error, dE):
            t1 = t1 + jacobi_update_t1_ai(r1, eps_o, eps_v)
            t2 = t2 + jacobi_update_t2_abij(r2, eps_o, eps_v)
            t1, t2 = diis.extrapolate([t1, t2], [r1, r2])
            tau = make_tau(t1, t2)
        else:
            converged = True
            break
        r1 = compute_cs_ccsd_r1(t1, t2, tau, ints)
        r2 = compute_cs_ccsd_r2(t1, t2, tau, ints)
        it += 1
    return SolveResult(E1, t1, t2, it, converged, history)


def ccsd_energy(ints: Integrals, t1, t2):
    """Standard closed-shell CCSD energy 2 f_ia t_ai + (2 g_ijab - g_ijba) tau_abij
    (the r = 0 limit of the residual-augmented functional of ccsd.h:377-379)."""
    tau = make_tau(t1, t2)
    g = ints.Gijab.transpose(2, 3, 0, 1)
    return 2.0 * float(np.vdot(ints.Fia.T, t1)) + float(np.vdot(g, 2.0 * tau - tau.transpose(1, 0, 2, 3)))


def flop_count(o, v):
    """Algorithmic FLOPs of one standard-method residual (no symmetry used)."""
    return 2 * o**2 * v**4 + 12 * o**3 * v**3 + 4 * o**4 * v**2 + 14 * o**2 * v**3 + 18 * o**3 * v**2
