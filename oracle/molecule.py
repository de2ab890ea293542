"""Molecular inputs for the CCSD oracle: Gaussian basis sets, one- and two-electron
integrals, closed-shell RHF and the MO integral blocks the CCSD solver consumes.

TEST INFRASTRUCTURE ONLY.  Like the rest of ``oracle/`` this module is a checker:
it turns the reference's molecular validation inputs (a geometry, a basis name,
frozen-core choice) into the MO integrals and orbital energies that MPQC's
``CCSD::compute_ccsd`` receives, so that the CCSD oracle -- and through it the
GPU solver -- can be compared with the reference's own recorded energies.  The
product never imports it.

What it restates (paths relative to the MPQC source tree):
  src/mpqc/chemistry/molecule/molecule.cpp:85-92   xyz in Angstrom -> Bohr with the
      units system of the input (2010 CODATA Bohr radius, units.h:97-104)
  src/mpqc/chemistry/qc/lcao/scf/rhf.h             closed-shell Roothaan-Hall SCF
  src/mpqc/chemistry/qc/lcao/wfn/lcao_wfn.h:43-70  frozen core (1 core orbital per
      first-row atom: "Frozen Core: 2 electrons" in the water outputs)
  src/mpqc/chemistry/qc/lcao/expression/...        MO blocks <ij|ab>, <ij|kl>, <ia|jb>,
      <ij|ka>, <ia|bc>, <ab|cd> and the Fock blocks, in annotation index order

The integrals themselves come from Libint2 in the reference (not part of the MPQC
tree).  Here they are computed with the McMurchie-Davidson scheme (L. E.
McMurchie and E. R. Davidson, J. Comput. Phys. 26, 218 (1978)): Hermite
expansion coefficients E_t^{ij}, Hermite Coulomb integrals R_tuv from the Boys
function, kinetic energy by the Gaussian derivative rule.  Basis sets are
Pople 6-31G (R. Ditchfield, W. J. Hehre, J. A. Pople, J. Chem. Phys. 54, 724
(1971); W. J. Hehre, R. Ditchfield, J. A. Pople, J. Chem. Phys. 56, 2257 (1972))
and Dunning cc-pVDZ (T. H. Dunning, J. Chem. Phys. 90, 1007 (1989)), H and O
only, with spherical d functions (cc-pVDZ water has 24 functions).

Energies are independent of how each contracted function is normalised, so the
AO matrices are simply rescaled to unit overlap diagonal at the end.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
from scipy.special import gammainc, gamma as gamma_fn

# 2010 CODATA Bohr radius in Angstrom (units.h:97-104 of the reference).
BOHR_ANGSTROM_2010 = 0.52917721092

Z_OF = {"H": 1, "O": 8}
# Core orbitals frozen per atom when frozen_core is on (first-row: 1s).
N_CORE_OF = {"H": 0, "O": 1}

# Each shell: (l, [(exponent, coefficient), ...]).  SP shells are split into an
# S and a P shell with shared exponents.
BASIS_SETS = {
    "6-31G": {
        "H": [
            (0, [(18.7311370, 0.03349460), (2.8253937, 0.23472695), (0.6401217, 0.81375733)]),
            (0, [(0.1612778, 1.0)]),
        ],
        "O": [
            (0, [(5484.67170, 0.00183110), (825.234950, 0.0139501), (188.046960, 0.0684451),
                 (52.9645000, 0.2327143), (16.8975700, 0.4701930), (5.79963530, 0.3585209)]),
            (0, [(15.5396160, -0.1107775), (3.59993360, -0.1480263), (1.01376180, 1.1307670)]),
            (1, [(15.5396160, 0.0708743), (3.59993360, 0.3397528), (1.01376180, 0.7271586)]),
            (0, [(0.27000580, 1.0)]),
            (1, [(0.27000580, 1.0)]),
        ],
    },
    "cc-pVDZ": {
        "H": [
            (0, [(13.0100, 0.019685), (1.9620, 0.137977), (0.4446, 0.478148)]),
            (0, [(0.1220, 1.0)]),
            (1, [(0.7270, 1.0)]),
        ],
        "O": [
            (0, [(11720.0, 0.000710), (1759.0, 0.005470), (400.8, 0.027837), (113.7, 0.104800),
                 (37.03, 0.283062), (13.27, 0.448719), (5.025, 0.270952), (1.013, 0.015458)]),
            (0, [(11720.0, -0.000160), (1759.0, -0.001263), (400.8, -0.006267), (113.7, -0.025716),
                 (37.03, -0.070924), (13.27, -0.165411), (5.025, -0.116955), (1.013, 0.557368)]),
            (0, [(0.3023, 1.0)]),
            (1, [(17.70, 0.043018), (3.854, 0.228913), (1.046, 0.508728)]),
            (1, [(0.2753, 1.0)]),
            (2, [(1.185, 1.0)]),
        ],
    },
}
# Pople polarisation shells (Hariharan & Pople 1973): Cartesian d on O
# (exponent 0.8) for 6-31G*, plus p on H (exponent 1.1) for 6-31G**.
BASIS_SETS["6-31G*"] = {"H": BASIS_SETS["6-31G"]["H"], "O": BASIS_SETS["6-31G"]["O"] + [(2, [(0.8, 1.0)])]}
BASIS_SETS["6-31G**"] = {"H": BASIS_SETS["6-31G"]["H"] + [(1, [(1.1, 1.0)])], "O": BASIS_SETS["6-31G*"]["O"]}


def cartesian_components(l):
    """(i, j, k) with i+j+k = l, x-major order."""
    return [(i, j, l - i - j) for i in range(l, -1, -1) for j in range(l - i, -1, -1)]


@dataclass
class Shell:
    l: int
    center: np.ndarray     # (3,) Bohr
    exps: np.ndarray       # (n,)
    coefs: np.ndarray      # (n,) contraction coefficient x primitive norm of x^l
    pure: bool             # spherical (l = 2 only needs it here)

    @property
    def ncart(self):
        return (self.l + 1) * (self.l + 2) // 2

    @property
    def nfunc(self):
        return 2 * self.l + 1 if (self.pure and self.l >= 2) else self.ncart


@dataclass
class Molecule:
    symbols: list
    coords: np.ndarray     # (natom, 3) Bohr

    @classmethod
    def from_xyz_text(cls, text, units_angstrom=BOHR_ANGSTROM_2010):
        lines = [ln.split() for ln in text.strip().splitlines()]
        n = int(lines[0][0])
        rows = [r for r in lines[1:] if len(r) >= 4][:n]
        sym = [r[0] for r in rows]
        xyz = np.array([[float(x) for x in r[1:4]] for r in rows]) / units_angstrom
        return cls(sym, xyz)

    def nuclear_repulsion(self):
        e = 0.0
        for a in range(len(self.symbols)):
            for b in range(a):
                e += Z_OF[self.symbols[a]] * Z_OF[self.symbols[b]] / np.linalg.norm(
                    self.coords[a] - self.coords[b])
        return e

    def n_electrons(self, charge=0):
        return sum(Z_OF[s] for s in self.symbols) - charge

    def n_frozen_core(self):
        return sum(N_CORE_OF[s] for s in self.symbols)


def build_shells(mol: Molecule, basis: str):
    pure = basis.startswith("cc-")
    shells = []
    for sym, c in zip(mol.symbols, mol.coords):
        for l, prims in BASIS_SETS[basis][sym]:
            e = np.array([p[0] for p in prims])
            d = np.array([p[1] for p in prims])
            norm = (2 * e / np.pi) ** 0.75 * (4 * e) ** (l / 2) / math.sqrt(
                max(1, _dfact(2 * l - 1)))
            shells.append(Shell(l, np.array(c, dtype=float), e, d * norm, pure))
    return shells


def _dfact(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


# ---------------------------------------------------------------------------
# McMurchie-Davidson building blocks
# ---------------------------------------------------------------------------

def hermite_E(la, lb, a, b, XAB):
    """E[i, j, t, pa, pb]: 1-D Hermite expansion coefficients of the product of
    x_A^i e^{-a x_A^2} and x_B^j e^{-b x_B^2} (i <= la, j <= lb, t <= i+j)."""
    p = a[:, None] + b[None, :]
    mu = a[:, None] * b[None, :] / p
    XPA = -b[None, :] / p * XAB
    XPB = a[:, None] / p * XAB
    E = np.zeros((la + 1, lb + 1, la + lb + 2) + p.shape)
    E[0, 0, 0] = np.exp(-mu * XAB * XAB)
    half_p = 0.5 / p
    for i in range(la + 1):
        for j in range(lb + 1):
            if i == 0 and j == 0:
                continue
            if i > 0:
                src, X, ii, jj = E[i - 1, j], XPA, i - 1, j
            else:
                src, X, ii, jj = E[i, j - 1], XPB, i, j - 1
            for t in range(ii + jj + 2):
                v = X * src[t]
                if t > 0:
                    v = v + half_p * src[t - 1]
                if t + 1 <= ii + jj:
                    v = v + (t + 1) * src[t + 1]
                E[i, j, t] = v
    return E


def boys(nmax, T):
    """F_n(T) for n = 0..nmax (array over T): the Boys function
    F_n(T) = int_0^1 u^{2n} exp(-T u^2) du, from the regularised lower incomplete
    gamma function for T >= 1 and its Taylor series below."""
    T = np.asarray(T, dtype=float)
    out = np.empty((nmax + 1,) + T.shape)
    small = T < 1.0
    Ts = np.where(small, T, 0.0)
    Tl = np.where(small, 1.0, T)
    for n in range(nmax + 1):
        # series: sum_k (-T)^k / (k! (2n + 2k + 1)), 30 terms reach 1e-17 at T = 1
        acc = np.zeros_like(Ts)
        term = np.ones_like(Ts)
        for k in range(30):
            acc = acc + term / (2 * n + 2 * k + 1)
            term = term * (-Ts) / (k + 1)
        big = gamma_fn(n + 0.5) * gammainc(n + 0.5, Tl) / (2.0 * Tl ** (n + 0.5))
        out[n] = np.where(small, acc, big)
    return out


def hermite_R(L, alpha, PQ):
    """R[t, u, v, ...] = R^0_{tuv}(alpha, PQ) for t+u+v <= L (zero elsewhere)."""
    X, Y, Z = PQ[..., 0], PQ[..., 1], PQ[..., 2]
    T = alpha * (X * X + Y * Y + Z * Z)
    F = boys(L, T)
    shape = alpha.shape
    # Rn[n][(t,u,v)] built from total order 0 up
    Rn = {}
    m2a = -2.0 * alpha
    for n in range(L + 1):
        Rn[(n, 0, 0, 0)] = m2a ** n * F[n]
    for tot in range(1, L + 1):
        for n in range(L - tot + 1):
            for t in range(tot + 1):
                for u in range(tot - t + 1):
                    v = tot - t - u
                    if t > 0:
                        val = X * Rn[(n + 1, t - 1, u, v)]
                        if t > 1:
                            val = val + (t - 1) * Rn[(n + 1, t - 2, u, v)]
                    elif u > 0:
                        val = Y * Rn[(n + 1, t, u - 1, v)]
                        if u > 1:
                            val = val + (u - 1) * Rn[(n + 1, t, u - 2, v)]
                    else:
                        val = Z * Rn[(n + 1, t, u, v - 1)]
                        if v > 1:
                            val = val + (v - 1) * Rn[(n + 1, t, u, v - 2)]
                    Rn[(n, t, u, v)] = val
    R = np.zeros((L + 1, L + 1, L + 1) + shape)
    for (n, t, u, v), val in Rn.items():
        if n == 0:
            R[t, u, v] = val
    return R


def _pair_E(sa: Shell, sb: Shell, extra_b=0):
    """3-D Hermite coefficients of a shell pair, one array per axis."""
    AB = sa.center - sb.center
    return [hermite_E(sa.l, sb.l + extra_b, sa.exps, sb.exps, AB[k]) for k in range(3)]


def _pair_hermite(sa: Shell, sb: Shell):
    """Eab[ca, cb, t, u, v, pa, pb] with contraction coefficients folded in."""
    Ex, Ey, Ez = _pair_E(sa, sb)
    L = sa.l + sb.l
    ca, cb = cartesian_components(sa.l), cartesian_components(sb.l)
    na, nb = len(sa.exps), len(sb.exps)
    out = np.zeros((len(ca), len(cb), L + 1, L + 1, L + 1, na, nb))
    for A, (ia, ja, ka) in enumerate(ca):
        for B, (ib, jb, kb) in enumerate(cb):
            ex = Ex[ia, ib, :ia + ib + 1]
            ey = Ey[ja, jb, :ja + jb + 1]
            ez = Ez[ka, kb, :ka + kb + 1]
            out[A, B, :ia + ib + 1, :ja + jb + 1, :ka + kb + 1] = (
                ex[:, None, None] * ey[None, :, None] * ez[None, None, :])
    out *= sa.coefs[:, None] * sb.coefs[None, :]
    return out


def _pure_matrix(l):
    """Rows: functions spanning the real solid harmonics of degree l, in terms of
    the Cartesian components of ``cartesian_components(l)``."""
    if l < 2:
        return np.eye((l + 1) * (l + 2) // 2)
    assert l == 2
    # xx, xy, xz, yy, yz, zz -> xy, yz, 2zz-xx-yy, xz, xx-yy
    return np.array([
        [0, 1, 0, 0, 0, 0],
        [0, 0, 0, 0, 1, 0],
        [-1, 0, 0, -1, 0, 2],
        [0, 0, 1, 0, 0, 0],
        [1, 0, 0, -1, 0, 0],
    ], dtype=float)


def _transform(shells):
    blocks = [(_pure_matrix(s.l) if (s.pure and s.l >= 2) else np.eye(s.ncart)) for s in shells]
    nc = sum(b.shape[1] for b in blocks)
    nf = sum(b.shape[0] for b in blocks)
    Tm = np.zeros((nf, nc))
    r = c = 0
    for b in blocks:
        Tm[r:r + b.shape[0], c:c + b.shape[1]] = b
        r += b.shape[0]
        c += b.shape[1]
    return Tm


def one_electron(shells, mol: Molecule):
    """Cartesian S, T, V over all shells (before the spherical transform)."""
    offs = np.cumsum([0] + [s.ncart for s in shells])
    n = offs[-1]
    S = np.zeros((n, n))
    Tk = np.zeros((n, n))
    V = np.zeros((n, n))
    for A, sa in enumerate(shells):
        for B, sb in enumerate(shells):
            Ex, Ey, Ez = _pair_E(sa, sb, extra_b=2)
            p = sa.exps[:, None] + sb.exps[None, :]
            b = sb.exps[None, :]
            sq = np.sqrt(np.pi / p)
            # 1-D overlaps S1[i, j] and kinetic T1[i, j]
            def s1(E, i, j):
                return E[i, j, 0] * sq if j >= 0 else 0.0
            P = (sa.exps[:, None, None] * sa.center + sb.exps[None, :, None] * sb.center) / p[..., None]
            L = sa.l + sb.l
            Rc = []
            for zc, cc in zip(mol.symbols, mol.coords):
                Rc.append((Z_OF[zc], hermite_R(L, p, P - cc)))
            cw = sa.coefs[:, None] * sb.coefs[None, :]
            for a_i, (ia, ja, ka) in enumerate(cartesian_components(sa.l)):
                for b_i, (ib, jb, kb) in enumerate(cartesian_components(sb.l)):
                    sx, sy, sz = s1(Ex, ia, ib), s1(Ey, ja, jb), s1(Ez, ka, kb)

                    def t1(E, i, j):
                        v = -2 * b * b * s1(E, i, j + 2) + b * (2 * j + 1) * s1(E, i, j)
                        if j >= 2:
                            v = v - 0.5 * j * (j - 1) * s1(E, i, j - 2)
                        return v
                    tx, ty, tz = t1(Ex, ia, ib), t1(Ey, ja, jb), t1(Ez, ka, kb)
                    i0, j0 = offs[A] + a_i, offs[B] + b_i
                    S[i0, j0] = np.sum(cw * sx * sy * sz)
                    Tk[i0, j0] = np.sum(cw * (tx * sy * sz + sx * ty * sz + sx * sy * tz))
                    acc = 0.0
                    for Zc, R in Rc:
                        h = np.zeros_like(p)
                        for t in range(ia + ib + 1):
                            for u in range(ja + jb + 1):
                                for v in range(ka + kb + 1):
                                    h = h + Ex[ia, ib, t] * Ey[ja, jb, u] * Ez[ka, kb, v] * R[t, u, v]
                        acc -= Zc * np.sum(cw * 2 * np.pi / p * h)
                    V[i0, j0] = acc
    return S, Tk, V


def two_electron(shells):
    """Cartesian (ab|cd) over all shells, 8-fold symmetry, McMurchie-Davidson."""
    offs = np.cumsum([0] + [s.ncart for s in shells])
    n = offs[-1]
    G = np.zeros((n, n, n, n))
    ns = len(shells)
    pairs = [(a, b) for a in range(ns) for b in range(a + 1)]
    herm = {}
    info = {}
    for a, b in pairs:
        sa, sb = shells[a], shells[b]
        herm[(a, b)] = _pair_hermite(sa, sb)
        p = sa.exps[:, None] + sb.exps[None, :]
        P = (sa.exps[:, None, None] * sa.center + sb.exps[None, :, None] * sb.center) / p[..., None]
        info[(a, b)] = (p, P)
    for ip, (a, b) in enumerate(pairs):
        Eab = herm[(a, b)]
        p, P = info[(a, b)]
        Lab = shells[a].l + shells[b].l
        for (c, d) in pairs[:ip + 1]:
            Ecd = herm[(c, d)]
            q, Q = info[(c, d)]
            Lcd = shells[c].l + shells[d].l
            pp = p[:, :, None, None]
            qq = q[None, None, :, :]
            alpha = pp * qq / (pp + qq)
            PQ = P[:, :, None, None, :] - Q[None, None, :, :, :]
            R = hermite_R(Lab + Lcd, alpha, PQ)
            pref = 2 * np.pi ** 2.5 / (pp * qq * np.sqrt(pp + qq))
            h1 = np.arange(Lab + 1)
            h2 = np.arange(Lcd + 1)
            sgn = (-1.0) ** (h2[:, None, None] + h2[None, :, None] + h2[None, None, :])
            It = (h1[:, None, None, None, None, None] + h2[None, None, None, :, None, None])
            Iu = (h1[None, :, None, None, None, None] + h2[None, None, None, None, :, None])
            Iv = (h1[None, None, :, None, None, None] + h2[None, None, None, None, None, :])
            Rb = R[It, Iu, Iv] * pref  # (t,u,v,x,y,z, pa,pb,pc,pd)
            Es = Ecd * sgn[None, None, :, :, :, None, None]
            blk = np.einsum("ABtuvij,CDxyzkl,tuvxyzijkl->ABCD", Eab, Es, Rb, optimize=True)
            sa, sb, sc, sd = (slice(offs[s], offs[s + 1]) for s in (a, b, c, d))
            G[sa, sb, sc, sd] = blk
            G[sb, sa, sc, sd] = blk.transpose(1, 0, 2, 3)
            G[sa, sb, sd, sc] = blk.transpose(0, 1, 3, 2)
            G[sb, sa, sd, sc] = blk.transpose(1, 0, 3, 2)
            G[sc, sd, sa, sb] = blk.transpose(2, 3, 0, 1)
            G[sd, sc, sa, sb] = blk.transpose(3, 2, 0, 1)
            G[sc, sd, sb, sa] = blk.transpose(2, 3, 1, 0)
            G[sd, sc, sb, sa] = blk.transpose(3, 2, 1, 0)
    return G


def ao_integrals(mol: Molecule, basis: str):
    """S, H = T + V and (mu nu|la si) in the (spherical where required) AO basis,
    each function scaled to unit self-overlap."""
    shells = build_shells(mol, basis)
    S, Tk, V = one_electron(shells, mol)
    G = two_electron(shells)
    Tm = _transform(shells)
    S = Tm @ S @ Tm.T
    H = Tm @ (Tk + V) @ Tm.T
    G = np.einsum("pa,qb,rc,sd,abcd->pqrs", Tm, Tm, Tm, Tm, G, optimize=True)
    d = 1.0 / np.sqrt(np.diag(S))
    S = S * d[:, None] * d[None, :]
    H = H * d[:, None] * d[None, :]
    G = G * d[:, None, None, None] * d[None, :, None, None] * d[None, None, :, None] * d[None, None, None, :]
    return S, H, G


# ---------------------------------------------------------------------------
# Closed-shell RHF (Roothaan-Hall with Pulay DIIS on FDS - SDF)
# ---------------------------------------------------------------------------

@dataclass
class RHFResult:
    energy: float
    e_nuc: float
    C: np.ndarray
    eps: np.ndarray
    F: np.ndarray
    nocc: int
    iters: int


def rhf(S, H, G, nocc, e_nuc, conv=1e-13, max_iter=200, n_diis=8):
    w, U = np.linalg.eigh(S)
    X = U @ np.diag(w ** -0.5) @ U.T
    e, Cp = np.linalg.eigh(X.T @ H @ X)
    C = X @ Cp
    D = C[:, :nocc] @ C[:, :nocc].T
    Eold = 0.0
    fs, es = [], []
    for it in range(1, max_iter + 1):
        J = np.einsum("pqrs,rs->pq", G, D)
        K = np.einsum("prqs,rs->pq", G, D)
        F = H + 2 * J - K
        E = float(np.sum(D * (H + F))) + e_nuc
        err = F @ D @ S - S @ D @ F
        fs.append(F)
        es.append(err)
        if len(fs) > n_diis:
            fs.pop(0)
            es.pop(0)
        if abs(E - Eold) < conv and np.max(np.abs(err)) < 1e-10:
            break
        Eold = E
        m = len(fs)
        B = -np.ones((m + 1, m + 1))
        B[m, m] = 0.0
        for i in range(m):
            for j in range(m):
                B[i, j] = float(np.vdot(es[i], es[j]))
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        c = np.linalg.solve(B, rhs)[:m]
        Fd = sum(ci * fi for ci, fi in zip(c, fs))
        e, Cp = np.linalg.eigh(X.T @ Fd @ X)
        C = X @ Cp
        D = C[:, :nocc] @ C[:, :nocc].T
    # canonical orbitals of the converged Fock operator
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    C = X @ Cp
    return RHFResult(E, e_nuc, C, e, F, nocc, it)


# ---------------------------------------------------------------------------
# MO integral blocks in MPQC annotation order
# ---------------------------------------------------------------------------

def mo_blocks(scf: RHFResult, G, n_frozen):
    """The standard-method ``cc::Integrals`` members and the active orbital
    energies: Fia, Fij, Fab, Gijab=<ij|ab>, Gijkl, Giajb, Gijka, Giabc, Gabcd."""
    C = scf.C[:, n_frozen:]
    o = scf.nocc - n_frozen
    mo = np.einsum("pqrs,pi,qj,rk,sl->ijkl", G, C, C, C, C, optimize=True)  # (ij|kl)
    g = mo.transpose(0, 2, 1, 3)                                           # <ik|jl>
    Fmo = C.T @ scf.F @ C
    O, Vs = slice(0, o), slice(o, C.shape[1])
    blocks = dict(
        Fia=Fmo[O, Vs].copy(), Fij=Fmo[O, O].copy(), Fab=Fmo[Vs, Vs].copy(),
        Gijab=g[O, O, Vs, Vs].copy(), Gijkl=g[O, O, O, O].copy(), Giajb=g[O, Vs, O, Vs].copy(),
        Gijka=g[O, O, O, Vs].copy(), Giabc=g[O, Vs, Vs, Vs].copy(), Gabcd=g[Vs, Vs, Vs, Vs].copy(),
    )
    eps = np.diag(Fmo)
    return blocks, eps[:o].copy(), eps[o:].copy()


def mp2_energy(blocks, eps_o, eps_v):
    g = blocks["Gijab"]
    D = eps_o[:, None, None, None] + eps_o[None, :, None, None] - eps_v[None, None, :, None] - eps_v[None, None, None, :]
    t = g / D
    return float(np.sum(t * (2 * g - g.transpose(0, 1, 3, 2))))


def molecular_inputs(xyz_text, basis, frozen_core=True, charge=0):
    """xyz text -> (RHF result, MO blocks, eps_o, eps_v, n_frozen)."""
    mol = Molecule.from_xyz_text(xyz_text)
    S, H, G = ao_integrals(mol, basis)
    nocc = mol.n_electrons(charge) // 2
    scf = rhf(S, H, G, nocc, mol.nuclear_repulsion())
    nfz = mol.n_frozen_core() if frozen_core else 0
    blocks, eo, ev = mo_blocks(scf, G, nfz)
    return scf, blocks, eo, ev, nfz


# ---------------------------------------------------------------------------
# The same integrals from the C restatement (oracle/ints_ref.c), for systems
# too large for the Python shell loops above
# ---------------------------------------------------------------------------

def _ints_lib():
    import ctypes as C
    from . import build_ref
    lib = C.CDLL(str(build_ref.build()))
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    lib.oneint_sph.restype = C.c_int
    lib.oneint_sph.argtypes = [C.c_int, ip, dp, ip, dp, dp, C.c_int, C.c_int, dp, dp, dp, dp, dp]
    lib.eri_sph.restype = C.c_int
    lib.eri_sph.argtypes = [C.c_int, ip, dp, ip, dp, dp, C.c_int, dp]
    return lib


def _flat_shells(shells):
    import ctypes as C
    l = np.array([s.l for s in shells], dtype=np.int32)
    center = np.ascontiguousarray(np.array([s.center for s in shells], dtype=float))
    nprim = np.array([len(s.exps) for s in shells], dtype=np.int32)
    exps = np.ascontiguousarray(np.concatenate([s.exps for s in shells]))
    coefs = np.ascontiguousarray(np.concatenate([s.coefs for s in shells]))
    pure = int(any(s.pure for s in shells))
    ptr = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    return (len(shells), ptr(l, C.c_int), ptr(center, C.c_double), ptr(nprim, C.c_int),
            ptr(exps, C.c_double), ptr(coefs, C.c_double), pure), (l, center, nprim, exps, coefs)


def ao_integrals_c(mol: Molecule, basis: str, eri=True):
    """``ao_integrals`` computed by the C restatement: S, H = T + V and (if
    ``eri``) (mu nu|la si) in the spherical AO basis, each function scaled to
    unit self-overlap.  The ERI array is filled and rescaled in place."""
    import ctypes as C
    lib = _ints_lib()
    shells = build_shells(mol, basis)
    args, keep = _flat_shells(shells)
    nf = sum(s.nfunc for s in shells)
    Zn = np.array([float(Z_OF[s]) for s in mol.symbols])
    xyz = np.ascontiguousarray(mol.coords, dtype=float)
    S = np.zeros((nf, nf))
    Tk = np.zeros((nf, nf))
    V = np.zeros((nf, nf))
    dp = C.POINTER(C.c_double)
    lib.oneint_sph(*args, len(mol.symbols), Zn.ctypes.data_as(dp), xyz.ctypes.data_as(dp),
                   S.ctypes.data_as(dp), Tk.ctypes.data_as(dp), V.ctypes.data_as(dp))
    d = 1.0 / np.sqrt(np.diag(S))
    S = S * d[:, None] * d[None, :]
    H = (Tk + V) * d[:, None] * d[None, :]
    if not eri:
        return S, H, None
    G = np.empty((nf, nf, nf, nf))
    lib.eri_sph(*args, G.ctypes.data_as(dp))
    for p in range(nf):   # rescale in place, one slab at a time
        G[p] *= d[p] * (d[:, None, None] * d[None, :, None] * d[None, None, :])
    del keep
    return S, H, G


# ---------------------------------------------------------------------------
# Memory-lean variants for a few hundred basis functions (the same arithmetic)
# ---------------------------------------------------------------------------

def rhf_lean(S, H, G, nocc, e_nuc, conv=1e-13, max_iter=200, n_diis=8):
    """``rhf`` with the exchange matrix built one AO slab at a time, so that no
    N^4 temporary is made (G alone is 26.5 GB at N = 240)."""
    n = S.shape[0]

    def jk(D):
        J = (G.reshape(n * n, n * n) @ D.ravel()).reshape(n, n)
        K = np.empty((n, n))
        for p in range(n):
            K[p] = np.einsum("rqs,rs->q", G[p], D, optimize=True)
        return J, K

    w, U = np.linalg.eigh(S)
    X = U @ np.diag(w ** -0.5) @ U.T
    e, Cp = np.linalg.eigh(X.T @ H @ X)
    C = X @ Cp
    D = C[:, :nocc] @ C[:, :nocc].T
    Eold = 0.0
    fs, es = [], []
    for it in range(1, max_iter + 1):
        J, K = jk(D)
        F = H + 2 * J - K
        E = float(np.sum(D * (H + F))) + e_nuc
        err = F @ D @ S - S @ D @ F
        fs.append(F)
        es.append(err)
        if len(fs) > n_diis:
            fs.pop(0)
            es.pop(0)
        if abs(E - Eold) < conv and np.max(np.abs(err)) < 1e-10:
            break
        Eold = E
        m = len(fs)
        B = -np.ones((m + 1, m + 1))
        B[m, m] = 0.0
        for i in range(m):
            for j in range(m):
                B[i, j] = float(np.vdot(es[i], es[j]))
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        c = np.linalg.solve(B, rhs)[:m]
        Fd = sum(ci * fi for ci, fi in zip(c, fs))
        e, Cp = np.linalg.eigh(X.T @ Fd @ X)
        C = X @ Cp
        D = C[:, :nocc] @ C[:, :nocc].T
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    C = X @ Cp
    return RHFResult(E, e_nuc, C, e, F, nocc, it)


def mo_blocks_inplace(scf: RHFResult, G, n_frozen, chunk=8):
    """``mo_blocks`` for large N: the last three indices of G are transformed
    to the MO basis in place, one AO slab at a time (G is overwritten with
    (mu q|r s)); each block then takes the first index in chunks of its second
    index.  Needs all orbitals (number of MOs = N)."""
    C = scf.C
    n = C.shape[0]
    if C.shape[1] != n:
        raise ValueError("mo_blocks_inplace needs as many orbitals as basis functions")
    for mu in range(n):
        Y = G[mu] @ C                                  # (nu, la, s)
        Y = np.tensordot(C, Y, axes=([0], [1]))        # (r, nu, s)
        Y = np.tensordot(C, Y, axes=([0], [1]))        # (q, r, s)
        G[mu] = Y
    nocc = scf.nocc
    Ca = C[:, n_frozen:]
    o = nocc - n_frozen
    O, V = slice(n_frozen, nocc), slice(nocc, n)

    def block(P, Q, R, Sl):
        """<p r|q s> = (pq|rs) laid out [p][r][q][s] (MPQC annotation order)."""
        Cp = C[:, P]
        nq = Q.stop - Q.start
        out = np.empty((Cp.shape[1], R.stop - R.start, nq, Sl.stop - Sl.start))
        for q0 in range(0, nq, chunk):
            q1 = min(nq, q0 + chunk)
            Y = np.tensordot(Cp, G[:, Q.start + q0:Q.start + q1, R, Sl], axes=([0], [0]))  # (p, q, r, s)
            out[:, :, q0:q1, :] = Y.transpose(0, 2, 1, 3)
        return out

    Fmo = Ca.T @ scf.F @ Ca
    Oa, Va = slice(0, o), slice(o, Ca.shape[1])
    blocks = dict(
        Fia=Fmo[Oa, Va].copy(), Fij=Fmo[Oa, Oa].copy(), Fab=Fmo[Va, Va].copy(),
        Gijab=block(O, V, O, V), Gijkl=block(O, O, O, O), Giajb=block(O, O, V, V),
        Gijka=block(O, O, O, V), Giabc=block(O, V, V, V), Gabcd=block(V, V, V, V),
    )
    eps = np.diag(Fmo)
    return blocks, eps[:o].copy(), eps[o:].copy()


def df_factors_c(mol: Molecule, obs: str, dfbs: str):
    """Density-fitting factors of the two-electron integrals in the Coulomb
    metric: B[K, mu, nu] = sum_Q (P|Q)^(-1/2)[K,Q] (Q|mu nu), so that
    (mu nu|la si) ~ sum_K B[K,mu,nu] B[K,la,si] -- the "[df]" integrals of
    the reference's LCAO factory ((K|G|p q)[inv_sqr], lcao_factory.h) and of
    its RI-RHF.  The orbital basis is normalised as in ``ao_integrals_c``; the
    fitting functions' normalisation cancels.  The three- and two-centre
    integrals come from the C restatement's four-centre routine with a unit
    s function (exponent 0) next to each fitting function: (P 1|mu nu) and
    (P 1|Q 1).  Small molecules only: it fills an (N + Naux + 1)^4 array.
    Returns (S, H, B) with S and H of the orbital basis."""
    lib = _ints_lib()
    o_sh = build_shells(mol, obs)
    a_sh = build_shells(mol, dfbs)
    if any(s.pure and s.l >= 2 for s in a_sh) and any(not s.pure and s.l >= 2 for s in o_sh):
        raise ValueError("the C routine takes one pure flag: Cartesian d in the orbital basis "
                         "and spherical d in the fitting basis cannot be combined")
    pure = any(s.pure for s in a_sh)
    unit = Shell(0, np.array(mol.coords[0], dtype=float), np.array([0.0]), np.array([1.0]), pure)
    shells = [Shell(s.l, s.center, s.exps, s.coefs, pure) for s in o_sh + a_sh] + [unit]
    args, keep = _flat_shells(shells)
    nf = sum(s.nfunc for s in o_sh)
    na = sum(s.nfunc for s in a_sh)
    n = nf + na + 1
    G = np.empty((n, n, n, n))
    import ctypes as C
    lib.eri_sph(*args, G.ctypes.data_as(C.POINTER(C.c_double)))
    del keep
    S, H, _ = ao_integrals_c(mol, obs, eri=False)
    # ao_integrals_c scales each orbital-basis function to unit self-overlap;
    # the same factors from the raw overlap of the orbital shells
    S_raw = np.zeros((nf, nf))
    T_raw = np.zeros((nf, nf))
    V_raw = np.zeros((nf, nf))
    oargs, okeep = _flat_shells(o_sh)
    Zn = np.array([float(Z_OF[s]) for s in mol.symbols])
    xyz = np.ascontiguousarray(mol.coords, dtype=float)
    dp = C.POINTER(C.c_double)
    lib.oneint_sph(*oargs, len(mol.symbols), Zn.ctypes.data_as(dp), xyz.ctypes.data_as(dp),
                   S_raw.ctypes.data_as(dp), T_raw.ctypes.data_as(dp), V_raw.ctypes.data_as(dp))
    del okeep
    d = 1.0 / np.sqrt(np.diag(S_raw))
    P3 = G[nf:nf + na, n - 1, :nf, :nf] * d[None, :, None] * d[None, None, :]   # (P|mu nu)
    M = G[nf:nf + na, n - 1, nf:nf + na, n - 1]                                   # (P|Q)
    M = 0.5 * (M + M.T)
    w, U = np.linalg.eigh(M)
    Minv_half = (U / np.sqrt(w)) @ U.T
    B = np.einsum("kq,qmn->kmn", Minv_half, P3)
    return S, H, B
