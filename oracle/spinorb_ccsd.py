"""Independent spin-orbital CCSD (TEST INFRASTRUCTURE ONLY).

Used only to cross-check the spin-adapted closed-shell oracle in
``ccsd_ref.py``: both must give the same converged correlation energy on the
same spatial-orbital Fock matrix and integrals.  This is a restatement of the
published spin-orbital CCSD equations with the effective-Hamiltonian
intermediates of J. F. Stanton, J. Gauss, J. D. Watts and R. J. Bartlett,
J. Chem. Phys. 94, 4334 (1991), solved by plain Jacobi iterations.  It is
dense and O(n^6); keep it to a handful of orbitals.
"""
from __future__ import annotations

import numpy as np


def _es(spec, *ops):
    return np.einsum(spec, *ops, optimize=True)


def spin_orbital_hamiltonian(eps_o, eps_v, Gfull):
    """Spin-orbital Fock and antisymmetrised <pq||rs> from spatial data.

    ``Gfull[p,q,r,s] = <pq|rs>`` over the full spatial space (occupied first).
    Spin orbitals interleave alpha/beta: 2p (alpha), 2p+1 (beta)."""
    eps = np.concatenate([eps_o, eps_v])
    n = eps.size
    ns = 2 * n
    spin = np.arange(ns) % 2
    sp = np.arange(ns) // 2
    f = np.diag(np.repeat(eps, 2))
    g = Gfull[np.ix_(sp, sp, sp, sp)]
    same = (spin[:, None] == spin[None, :])
    pr = same[:, None, :, None]
    qs = same[None, :, None, :]
    ps = same[:, None, None, :]
    qr = same[None, :, :, None]
    direct = g * (pr & qs)
    exchange = g.transpose(0, 1, 3, 2) * (ps & qr)
    return f, direct - exchange


def solve(eps_o, eps_v, Gfull, tol=1e-12, max_iter=500):
    """Converged spin-orbital CCSD correlation energy."""
    o2 = 2 * eps_o.size
    f, g = spin_orbital_hamiltonian(eps_o, eps_v, Gfull)
    n = f.shape[0]
    o, v = slice(0, o2), slice(o2, n)
    fd = np.diag(f)
    Dia = fd[o][:, None] - fd[v][None, :]
    Dijab = fd[o][:, None, None, None] + fd[o][None, :, None, None] - fd[v][None, None, :, None] - fd[v][None, None, None, :]
    foo = f[o, o] - np.diag(fd[o])
    fvv = f[v, v] - np.diag(fd[v])
    fov = f[o, v]
    g_oovv = g[o, o, v, v]
    t1 = np.zeros((o2, n - o2))
    t2 = g_oovv / Dijab
    e_old = 0.0
    for _ in range(max_iter):
        tau_t = t2 + 0.5 * (_es("ia,jb->ijab", t1, t1) - _es("ib,ja->ijab", t1, t1))
        tau = t2 + _es("ia,jb->ijab", t1, t1) - _es("ib,ja->ijab", t1, t1)
        Fae = (fvv - 0.5 * _es("me,ma->ae", fov, t1) + _es("mf,mafe->ae", t1, g[o, v, v, v])
               - 0.5 * _es("mnaf,mnef->ae", tau_t, g_oovv))
        Fmi = (foo + 0.5 * _es("ie,me->mi", t1, fov) + _es("ne,mnie->mi", t1, g[o, o, o, v])
               + 0.5 * _es("inef,mnef->mi", tau_t, g_oovv))
        Fme = fov + _es("nf,mnef->me", t1, g_oovv)
        Wmnij = (g[o, o, o, o] + _es("je,mnie->mnij", t1, g[o, o, o, v])
                 - _es("ie,mnje->mnij", t1, g[o, o, o, v]) + 0.25 * _es("ijef,mnef->mnij", tau, g_oovv))
        Wabef = (g[v, v, v, v] - _es("mb,amef->abef", t1, g[v, o, v, v])
                 + _es("ma,bmef->abef", t1, g[v, o, v, v]) + 0.25 * _es("mnab,mnef->abef", tau, g_oovv))
        Wmbej = (g[o, v, v, o] + _es("jf,mbef->mbej", t1, g[o, v, v, v])
                 - _es("nb,mnej->mbej", t1, g[o, o, v, o])
                 - _es("jnfb,mnef->mbej", 0.5 * t2 + _es("jf,nb->jnfb", t1, t1), g_oovv))
        r1 = (fov.copy() + _es("ie,ae->ia", t1, Fae) - _es("ma,mi->ia", t1, Fmi)
              + _es("imae,me->ia", t2, Fme) - _es("nf,naif->ia", t1, g[o, v, o, v])
              - 0.5 * _es("imef,maef->ia", t2, g[o, v, v, v]) - 0.5 * _es("mnae,nmei->ia", t2, g[o, o, v, o]))
        Fbe = Fae - 0.5 * _es("mb,me->be", t1, Fme)
        Fmj = Fmi + 0.5 * _es("je,me->mj", t1, Fme)
        x = _es("ijae,be->ijab", t2, Fbe)
        r2 = g_oovv.copy() + x - x.transpose(0, 1, 3, 2)
        y = _es("imab,mj->ijab", t2, Fmj)
        r2 -= y - y.transpose(1, 0, 2, 3)
        r2 += 0.5 * _es("mnab,mnij->ijab", tau, Wmnij) + 0.5 * _es("ijef,abef->ijab", tau, Wabef)
        z = _es("imae,mbej->ijab", t2, Wmbej) - _es("ie,ma,mbej->ijab", t1, t1, g[o, v, v, o])
        r2 += z - z.transpose(1, 0, 2, 3) - z.transpose(0, 1, 3, 2) + z.transpose(1, 0, 3, 2)
        w = _es("ie,abej->ijab", t1, g[v, v, v, o])
        r2 += w - w.transpose(1, 0, 2, 3)
        u = _es("ma,mbij->ijab", t1, g[o, v, o, o])
        r2 -= u - u.transpose(0, 1, 3, 2)
        t1 = r1 / Dia
        t2 = r2 / Dijab
        e = (_es("ia,ia->", fov, t1) + 0.25 * _es("ijab,ijab->", g_oovv, t2)
             + 0.5 * _es("ijab,ia,jb->", g_oovv, t1, t1))
        if abs(e - e_old) < tol:
            return float(e)
        e_old = e
    raise RuntimeError("spin-orbital CCSD did not converge")
