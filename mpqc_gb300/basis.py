"""Gaussian basis sets for the SCF input producer (the data MPQC reads from
Libint2's basis library, src/mpqc/chemistry/qc/lcao/basis/basis.cpp:28,49).

Published contraction tables, hydrogen and oxygen:
  6-31G    R. Ditchfield, W. J. Hehre, J. A. Pople, J. Chem. Phys. 54, 724 (1971);
           W. J. Hehre, R. Ditchfield, J. A. Pople, J. Chem. Phys. 56, 2257 (1972)
  6-31G*   6-31G plus one Cartesian d shell on O (exponent 0.8), and
  6-31G**  6-31G* plus one p shell on H (exponent 1.1): P. C. Hariharan,
           J. A. Pople, Theor. Chim. Acta 28, 213 (1973)
  cc-pVDZ  T. H. Dunning, J. Chem. Phys. 90, 1007 (1989); spherical d shells
Each shell is (l, [(exponent, coefficient of the normalised primitive), ...]);
SP shells are listed as an S and a P shell with shared exponents.

Other elements and basis sets are not provided.  6-31G and cc-pVDZ are pinned
by the reference's recorded water energies; the polarised 6-31G sets have no
recorded reference energy and are checked against the oracle's chain only.
"""
from __future__ import annotations

import numpy as np

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
BASIS_SETS["6-31G*"] = {"H": BASIS_SETS["6-31G"]["H"], "O": BASIS_SETS["6-31G"]["O"] + [(2, [(0.8, 1.0)])]}
BASIS_SETS["6-31G**"] = {"H": BASIS_SETS["6-31G"]["H"] + [(1, [(1.1, 1.0)])], "O": BASIS_SETS["6-31G*"]["O"]}

# spherical d functions in the Dunning sets, Cartesian (6D) in the Pople sets
PURE = {"6-31G": False, "6-31G*": False, "6-31G**": False, "cc-pVDZ": True}

NUCLEAR_CHARGE = {"H": 1, "O": 8}
# core orbitals per atom frozen by frozen_core (first row: 1s), as
# src/mpqc/chemistry/qc/lcao/wfn/lcao_wfn.h:55 counts them
N_CORE = {"H": 0, "O": 1}


def shells_for(symbols, basis):
    """Flattened shell arrays for ``gbcc_basis``: atom, l, nprim, exps, coefs, pure."""
    if basis not in BASIS_SETS:
        raise KeyError(f"basis {basis!r} is not available (have: {sorted(BASIS_SETS)})")
    table = BASIS_SETS[basis]
    atom, ls, nprim, exps, coefs = [], [], [], [], []
    for a, sym in enumerate(symbols):
        if sym not in table:
            raise KeyError(f"element {sym!r} is not in the {basis} table")
        for l, prims in table[sym]:
            atom.append(a)
            ls.append(l)
            nprim.append(len(prims))
            exps.extend(p[0] for p in prims)
            coefs.extend(p[1] for p in prims)
    return (np.array(atom, dtype=np.int32), np.array(ls, dtype=np.int32), np.array(nprim, dtype=np.int32),
            np.array(exps, dtype=np.float64), np.array(coefs, dtype=np.float64), PURE[basis])


def n_functions(symbols, basis):
    pure = PURE[basis]
    return sum((2 * l + 1 if (pure and l == 2) else (l + 1) * (l + 2) // 2)
               for s in symbols for l, _ in BASIS_SETS[basis][s])
