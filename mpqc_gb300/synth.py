"""Seeded synthetic CCSD inputs: density-fitted integrals over the full MO space.

The synthetic doubles-residual workload (o occupied, v virtual, naux auxiliary
functions) is built as follows, with ``numpy.random.default_rng(seed)``:

* ``B[Q,p,q]`` over the full space (n = o + v), entries N(0, b_scale), symmetrised
  in (p,q) so the integrals carry the 8-fold permutational symmetry of real
  orbitals that the spin-adapted equations assume;
* ``<pq|rs> = (pr|qs) = sum_Q B[Q,p,r] B[Q,q,s]`` for every block
  (Gijab, Gijkl, Giajb, Gijka, Giabc, Gabcd), so all blocks are mutually
  consistent and (ab|cd) is positive semidefinite;
* canonical Fock: eps_occ ~ U(-1.5,-0.3), eps_virt ~ U(0.1,3.0), off-diagonal 0;
* amplitudes: t2 ~ N(0, t2_scale) symmetrised t2[a,b,i,j] = t2[b,a,j,i],
  t1 ~ N(0, t1_scale) (zero when t1_scale is 0);
* uneven tile boundaries drawn in [tile_min, tile_max] for the o and v ranges
  (the block-sparse tiling the reference would hand over; the dense device
  layout does not depend on it).

All tensors are returned in MPQC annotation order (see ``Inputs``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Inputs:
    o: int
    v: int
    eps_o: np.ndarray
    eps_v: np.ndarray
    Fia: np.ndarray      # [i,a]
    Fij: np.ndarray      # [i,j]
    Fab: np.ndarray      # [a,b]
    Gijab: np.ndarray    # [i,j,a,b] = <ij|ab>
    Gijkl: np.ndarray    # [i,j,k,l]
    Giajb: np.ndarray    # [i,a,j,b]
    Gijka: np.ndarray    # [i,j,k,a]
    Giabc: np.ndarray    # [i,a,b,c]
    Gabcd: np.ndarray    # [a,b,c,d]
    t1: np.ndarray       # [a,i]
    t2: np.ndarray       # [a,b,i,j]
    tiles_o: list
    tiles_v: list


def uneven_tiles(rng, n, lo, hi):
    """Tile boundaries [0, b1, ..., n] with every tile in [lo, hi] except a
    possibly shorter last one (a single tile when n <= hi)."""
    bounds = [0]
    while bounds[-1] < n:
        step = int(rng.integers(lo, hi + 1))
        bounds.append(min(n, bounds[-1] + step))
    return bounds


def make_df_factor(rng, naux, n, b_scale):
    x = rng.normal(0.0, b_scale, size=(naux, n, n))
    return (x + x.transpose(0, 2, 1)) * (0.5 ** 0.5)


def build_blocks(B, o, v):
    """All six <pq|rs> blocks from one DF factor over the full space."""
    Bo_o = B[:, :o, :o]
    Bo_v = B[:, :o, o:]
    Bv_v = B[:, o:, o:]

    def g(x, y):  # <pq|rs> = sum_Q x[Q,p,r] y[Q,q,s]
        return np.einsum("Qpr,Qqs->pqrs", x, y, optimize=True)

    return dict(
        Gijab=g(Bo_v, Bo_v),
        Gijkl=g(Bo_o, Bo_o),
        Giajb=g(Bo_o, Bv_v),
        Gijka=g(Bo_o, Bo_v),
        Giabc=g(Bo_v, Bv_v),
        Gabcd=g(Bv_v, Bv_v),
    )


def make_inputs(o, v, naux, seed=0, b_scale=0.05, t2_scale=1e-2, t1_scale=0.0,
                tile_min=20, tile_max=64):
    rng = np.random.default_rng(seed)
    n = o + v
    B = make_df_factor(rng, naux, n, b_scale)
    eps_o = np.sort(rng.uniform(-1.5, -0.3, size=o))
    eps_v = np.sort(rng.uniform(0.1, 3.0, size=v))
    t2 = rng.normal(0.0, t2_scale, size=(v, v, o, o))
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    t1 = rng.normal(0.0, t1_scale, size=(v, o)) if t1_scale > 0 else np.zeros((v, o))
    tiles_o = uneven_tiles(rng, o, tile_min, tile_max)
    tiles_v = uneven_tiles(rng, v, tile_min, tile_max)
    return inputs_from_factor(B, eps_o, eps_v, t1, t2, tiles_o, tiles_v)


def inputs_from_factor(B, eps_o, eps_v, t1, t2, tiles_o=None, tiles_v=None):
    """Inputs for a given DF factor B[Q,p,q] over the full space and Fock
    diagonal (canonical orbitals: Fia = 0, Fij/Fab diagonal)."""
    o, v = eps_o.size, eps_v.size
    return Inputs(
        o=o, v=v, eps_o=eps_o, eps_v=eps_v,
        Fia=np.zeros((o, v)), Fij=np.diag(eps_o), Fab=np.diag(eps_v),
        t1=t1, t2=t2,
        tiles_o=tiles_o if tiles_o is not None else [0, o],
        tiles_v=tiles_v if tiles_v is not None else [0, v],
        **build_blocks(B, o, v),
    )


def flop_count(o, v):
    """Algorithmic FLOPs of one standard-method R1+R2 residual, counted from
    the reference's contractions without exploiting any symmetry."""
    return (2 * o**2 * v**4 + 12 * o**3 * v**3 + 4 * o**4 * v**2
            + 14 * o**2 * v**3 + 18 * o**3 * v**2)
