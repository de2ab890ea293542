"""FP64 CPU oracle for the perturbative triples correction (T) of closed-shell
CCSD.

TEST INFRASTRUCTURE ONLY (tests/, bench.py's CPU legs); the product path never
imports it.

Restates the reference's "straight" (T) (src/mpqc/chemistry/qc/lcao/cc/
ccsd_t.h:1127-1167, with the denominator reduction CCSD_T_Reduce at
ccsd_t.h:2274-2333 and the integral getters at ccsd_t.h:2210-2244), in the
same MPQC annotation order as ccsd_ref.py:

    g_cjkl(c,j,k,l) = <jk|lc> = Gijka[j,k,l,c]        (get_aijk)
    g_dabi(d,a,b,i) = <id|ab> = Giabc[i,d,a,b]        (get_abci)
    g_abij(a,b,i,j) = <ij|ab> = Gijab[i,j,a,b]        (get_abij)

    t3(a,b,c,i,j,k) = g_dabi(d,a,b,i) t2(d,c,j,k) - g_cjkl(c,j,k,l) t2(a,b,i,l)
    t3 <- sum of t3 over the six simultaneous permutations of (a,i),(b,j),(c,k)
    v3(a,b,c,i,j,k) = g_abij(a,b,i,j) t1(c,k) + (b,c,a,j,k,i) + (a,c,b,i,k,j) terms
    E(T) = 1/3 sum (t3 + v3) (4 t3 + t3(abc,kij) + t3(abc,jki)
                              - 2 (t3(abc,kji) + t3(abc,ikj) + t3(abc,jik)))
                   / (e_i + e_j + e_k - e_a - e_b - e_c)

``triples_energy`` forms the full o^3 v^3 arrays (small systems only);
``triples_energy_by_triplet`` evaluates the same sum one occupied triplet at a
time with each triplet's terms written through the virtual-index
permutations that the permutational symmetry of t3 allows (t3(a,b,c,k,i,j) =
t3(b,c,a,i,j,k), ...), over i <= j <= k with multiplicities: the
arrangement the GPU evaluates, checked equal to the first.
"""
from __future__ import annotations

import numpy as np


def _es(spec, *ops):
    return np.einsum(spec, *ops, optimize=True)


def t3_v3(t1, t2, Gijab, Gijka, Giabc):
    """The connected (t3) and disconnected (v3) triples of ccsd_t.h:1139-1152."""
    g_dabi = Giabc.transpose(1, 2, 3, 0)        # g_dabi[d,a,b,i] = Giabc[i,d,a,b]
    g_cjkl = Gijka.transpose(3, 0, 1, 2)        # g_cjkl[c,j,k,l] = Gijka[j,k,l,c]
    g_abij = Gijab.transpose(2, 3, 0, 1)        # g_abij[a,b,i,j] = Gijab[i,j,a,b]
    x = _es("dabi,dcjk->abcijk", g_dabi, t2) - _es("cjkl,abil->abcijk", g_cjkl, t2)
    t3 = (x + x.transpose(0, 2, 1, 3, 5, 4) + x.transpose(2, 0, 1, 5, 3, 4) + x.transpose(2, 1, 0, 5, 4, 3)
          + x.transpose(1, 2, 0, 4, 5, 3) + x.transpose(1, 0, 2, 4, 3, 5))
    y = _es("abij,ck->abcijk", g_abij, t1)
    v3 = y + y.transpose(2, 0, 1, 5, 3, 4) + y.transpose(0, 2, 1, 3, 5, 4)
    return t3, v3


def triples_energy(t1, t2, Gijab, Gijka, Giabc, eps_o, eps_v):
    """E(T) of ccsd_t.h:1154-1166 (full arrays)."""
    t3, v3 = t3_v3(t1, t2, Gijab, Gijka, Giabc)
    w = (4.0 * t3 + t3.transpose(0, 1, 2, 4, 5, 3) + t3.transpose(0, 1, 2, 5, 3, 4)
         - 2.0 * (t3.transpose(0, 1, 2, 5, 4, 3) + t3.transpose(0, 1, 2, 3, 5, 4) + t3.transpose(0, 1, 2, 4, 3, 5)))
    d = (eps_o[None, None, None, :, None, None] + eps_o[None, None, None, None, :, None]
         + eps_o[None, None, None, None, None, :] - eps_v[:, None, None, None, None, None]
         - eps_v[None, :, None, None, None, None] - eps_v[None, None, :, None, None, None])
    return float(np.sum((t3 + v3) * w / d) / 3.0)


def triplet_blocks(t1, t2, Gijab, Gijka, Giabc, i, j, k):
    """W[a,b,c] = t3(a,b,c,i,j,k) and V[a,b,c] = v3(a,b,c,i,j,k) of one
    occupied triplet, each of the six permutation terms as one v^3 x v
    (or v^3 x o) contraction (the GEMMs of the GPU path)."""
    G = Giabc                                   # G[x,d,p,q] = <xd|pq>
    R = Gijka                                   # R[y,z,l,c] = <yz|lc>

    def xd(x, y, z):   # sum_d <xd|pq> t2(d,r,y,z) - sum_l <yz|lr> t2(p,q,x,l), as [p,q,r]
        return _es("dpq,dr->pqr", G[x], t2[:, :, y, z]) - _es("lr,pql->pqr", R[y, z], t2[:, :, x, :])

    W = (xd(i, j, k)                            # t3 term (a,b,c,i,j,k)
         + xd(i, k, j).transpose(0, 2, 1)       # (a,c,b,i,k,j)
         + xd(j, i, k).transpose(1, 0, 2)       # (b,a,c,j,i,k)
         + xd(j, k, i).transpose(2, 0, 1)       # (b,c,a,j,k,i): [b,c,a] -> [a,b,c]
         + xd(k, i, j).transpose(1, 2, 0)       # (c,a,b,k,i,j): [c,a,b] -> [a,b,c]
         + xd(k, j, i).transpose(2, 1, 0))      # (c,b,a,k,j,i)
    g = Gijab                                   # g[i,j,a,b] = <ij|ab>
    V = (_es("ab,c->abc", g[i, j], t1[:, k]) + _es("bc,a->abc", g[j, k], t1[:, i])
         + _es("ac,b->abc", g[i, k], t1[:, j]))
    return W, V


def triplet_energy(W, V, ei, ej, ek, eps_v):
    """The abc sum of one triplet: the occupied-index permutations of t3 read
    as virtual-index permutations of W (t3(abc,kij) = W[b,c,a], ...)."""
    Y = (4.0 * W + W.transpose(1, 2, 0) + W.transpose(2, 0, 1)
         - 2.0 * (W.transpose(2, 1, 0) + W.transpose(0, 2, 1) + W.transpose(1, 0, 2)))
    d = ei + ej + ek - eps_v[:, None, None] - eps_v[None, :, None] - eps_v[None, None, :]
    return float(np.sum((W + V) * Y / d))


def triples_energy_by_triplet(t1, t2, Gijab, Gijka, Giabc, eps_o, eps_v):
    """E(T) over i <= j <= k: a triplet's abc sum is the same for every
    ordering of (i, j, k), so each counts once per distinct permutation."""
    o = eps_o.size
    e = 0.0
    for i in range(o):
        for j in range(i, o):
            for k in range(j, o):
                mult = 6 if i < j < k else (1 if i == j == k else 3)
                W, V = triplet_blocks(t1, t2, Gijab, Gijka, Giabc, i, j, k)
                e += mult * triplet_energy(W, V, eps_o[i], eps_o[j], eps_o[k], eps_v)
    return e / 3.0
