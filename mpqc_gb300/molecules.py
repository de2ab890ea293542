"""Molecular geometries of the benchmark systems (Angstrom) and units.

* ``water()``: O at (0, 0, 0.1173), H at (0, +-0.7572, -0.4692) Angstrom
  (r(OH) = 0.9578 Angstrom, 104.5 degrees), the single-water benchmark system.
* ``water_cluster(n, seed)``: (H2O)n with the waters' oxygens on the first n of
  ten sites -- the eight corners of a cube of edge 2.9 Angstrom, then the
  centres of its bottom and top faces -- each water with the geometry above,
  rotated by a rotation drawn uniformly (a normalised Gaussian quaternion)
  from ``numpy.random.default_rng(seed)``.  A draw that brings two atoms of
  different waters closer than ``min_contact`` is drawn again from the same
  generator, so the clusters have no fused atoms; the result is a fixed
  function of (n, seed).

Coordinates go to the integrals in Bohr with the 2010 CODATA Bohr radius, as
the reference's inputs request ("units": "2010CODATA";
src/mpqc/chemistry/units/units.h:97-104 and molecule.cpp:85-92).
"""
from __future__ import annotations

import numpy as np

BOHR_ANGSTROM_2010 = 0.52917721092

WATER = (("O", (0.0, 0.0, 0.1173)), ("H", (0.0, 0.7572, -0.4692)), ("H", (0.0, -0.7572, -0.4692)))
CUBE_EDGE = 2.9


def water():
    return [s for s, _ in WATER], np.array([x for _, x in WATER], dtype=float)


def cluster_sites(edge=CUBE_EDGE):
    corners = [(x, y, z) for x in (0.0, edge) for y in (0.0, edge) for z in (0.0, edge)]
    faces = [(0.5 * edge, 0.5 * edge, 0.0), (0.5 * edge, 0.5 * edge, edge)]
    return np.array(corners + faces, dtype=float)


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def water_cluster(n, seed=0, edge=CUBE_EDGE, min_contact=1.4, max_draws=10000):
    """(symbols, coordinates in Angstrom) of (H2O)n, 1 <= n <= 10."""
    sites = cluster_sites(edge)
    if not 1 <= n <= len(sites):
        raise ValueError(f"n must be 1..{len(sites)}")
    rng = np.random.default_rng(seed)
    sym0, geo0 = water()
    geo0 = geo0 - geo0[0]  # oxygen at the origin
    symbols, coords = [], []
    for k in range(n):
        for _ in range(max_draws):
            mol = geo0 @ random_rotation(rng).T + sites[k]
            if not coords:
                break
            prev = np.array(coords)
            d = np.linalg.norm(mol[:, None, :] - prev[None, :, :], axis=-1)
            if d.min() >= min_contact:
                break
        else:
            raise RuntimeError("no orientation without close contacts found")
        symbols.extend(sym0)
        coords.extend(mol.tolist())
    return symbols, np.array(coords)


def xyz_text(symbols, coords, comment=""):
    lines = [str(len(symbols)), comment]
    lines += [f"{s} {x:.10f} {y:.10f} {z:.10f}" for s, (x, y, z) in zip(symbols, coords)]
    return "\n".join(lines) + "\n"


def to_bohr(coords_angstrom):
    return np.asarray(coords_angstrom, dtype=float) / BOHR_ANGSTROM_2010
