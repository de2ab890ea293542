"""CPU checks of the SCF input producer: the host eigensolver against numpy,
argument validation of gbcc_scf_create (no GPU needed: inputs are checked
before any CUDA call), the product's basis tables against the oracle's, the
C restatement of the integrals against the Python one, and the index
arithmetic the ERI kernel uses to enumerate shell quartets."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from mpqc_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.mark.parametrize("n,kind", [(1, "rand"), (2, "rand"), (7, "rand"), (48, "rand"), (240, "rand"),
                                    (30, "degenerate"), (25, "diagonal"), (64, "clustered")])
def test_eigh_matches_numpy(lib, n, kind):
    rng = np.random.default_rng(n)
    if kind == "rand":
        A = rng.normal(size=(n, n))
        A = A + A.T
    elif kind == "degenerate":
        Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
        w0 = np.repeat([-2.0, 0.5, 3.0], n // 3)
        A = (Q * w0) @ Q.T
    elif kind == "diagonal":
        A = np.diag(rng.normal(size=n))
    else:
        Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
        w0 = 1.0 + 1e-9 * rng.normal(size=n)
        A = (Q * w0) @ Q.T
    A = np.ascontiguousarray(0.5 * (A + A.T))
    w, V = np.empty(n), np.empty((n, n))
    assert lib.gbcc_testing_eigh(n, A.ctypes.data, w.ctypes.data, V.ctypes.data) == 0
    wr = np.linalg.eigvalsh(A)
    scale = max(1.0, float(np.max(np.abs(wr))))
    assert np.max(np.abs(w - wr)) < 1e-12 * scale * max(1, n) ** 0.5
    assert np.all(np.diff(w) >= 0)
    assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-12 * max(1, n)
    assert np.max(np.abs(A @ V - V * w)) < 1e-11 * scale * max(1, n) ** 0.5


def _scf_args(symbols, coords_bohr, basis):
    from mpqc_gb300 import _lib as L, basis as B
    zn = np.array([float(B.NUCLEAR_CHARGE[s]) for s in symbols])
    xyz = np.ascontiguousarray(coords_bohr, dtype=float)
    atom, ls, nprim, exps, coefs, pure = B.shells_for(symbols, basis)
    keep = [zn, xyz, atom, ls, nprim, exps, coefs]
    mol = L.Molecule(len(symbols), zn.ctypes.data, xyz.ctypes.data, 0)
    bas = L.Basis(len(ls), atom.ctypes.data, ls.ctypes.data, nprim.ctypes.data, exps.ctypes.data,
                  coefs.ctypes.data, int(pure))
    cfg = L.ScfConfig()
    return mol, bas, cfg, keep


def test_scf_create_rejects_bad_input(lib):
    from mpqc_gb300 import _lib as L, molecules
    sym, xyz = molecules.water()
    mol, bas, cfg, keep = _scf_args(sym, molecules.to_bohr(xyz), "cc-pVDZ")
    lib.gbcc_scf_config_default(C.byref(cfg))
    assert cfg.max_iter == 30 and cfg.n_diis == 8 and cfg.threshold == 1e-11
    h = C.c_void_p()

    def create():
        return lib.gbcc_scf_create(C.byref(h), C.byref(mol), C.byref(bas), C.byref(cfg))

    mol.mol_charge = 1                       # odd electron count
    assert create() == L.GBCC_ERR_INVALID_ARG and not h.value
    assert b"even" in lib.gbcc_last_scf_error(None)
    mol.mol_charge = 0
    ls = keep[3]
    ls[0] = 3                                # f shell
    assert create() == L.GBCC_ERR_INVALID_ARG and b"l = 2" in lib.gbcc_last_scf_error(None)
    ls[0] = 0
    keep[5][0] = 0.0                         # zero exponent
    assert create() == L.GBCC_ERR_INVALID_ARG
    keep[5][0] = 11720.0
    keep[1][1] = keep[1][0]                  # two nuclei at one point
    assert create() == L.GBCC_ERR_INVALID_ARG and b"same position" in lib.gbcc_last_scf_error(None)
    keep[1][1] = molecules.to_bohr(xyz)[1]
    cfg.max_iter = 0
    assert create() == L.GBCC_ERR_INVALID_ARG
    assert lib.gbcc_scf_destroy(None) == L.GBCC_OK


def test_basis_tables_match_the_oracle():
    from mpqc_gb300 import basis as B
    from oracle import molecule as M
    for name in ("6-31G", "6-31G*", "6-31G**", "cc-pVDZ"):
        for el in ("H", "O"):
            assert B.BASIS_SETS[name][el] == M.BASIS_SETS[name][el], (name, el)


def test_c_integrals_match_the_python_oracle():
    from oracle import molecule as M
    from mpqc_gb300 import molecules
    sym, xyz = molecules.water()
    mol = M.Molecule(sym, molecules.to_bohr(xyz))
    # 6-31G* has Cartesian (6D) d shells: the C oracle's transform buffers
    # must hold six functions per d shell, not five
    for basis in ("6-31G", "6-31G*", "cc-pVDZ"):
        S, H, G = M.ao_integrals(mol, basis)
        S2, H2, G2 = M.ao_integrals_c(mol, basis)
        assert np.max(np.abs(S - S2)) < 1e-13
        assert np.max(np.abs(H - H2)) < 1e-12
        assert np.max(np.abs(G - G2)) < 1e-13


def _decode_triangle(q):
    """The ERI kernel's quartet decode for bra and ket pairs of one class."""
    ip = int((np.sqrt(8.0 * q + 1.0) - 1.0) * 0.5)
    while ip * (ip + 1) // 2 > q:
        ip -= 1
    while (ip + 1) * (ip + 2) // 2 <= q:
        ip += 1
    return ip, q - ip * (ip + 1) // 2


def test_eri_quartet_enumeration_covers_each_pair_of_pairs_once():
    """Every unordered pair of shell pairs is one quartet, bra class >= ket
    class, and the triangular decode stays inside the class's pair range
    (checked at (H2O)10 / cc-pVDZ sizes: 120 shells, 7260 pairs)."""
    from mpqc_gb300 import basis as B, molecules
    sym, _ = molecules.water_cluster(10, seed=0)
    _, ls, _, _, _, _ = B.shells_for(sym, "cc-pVDZ")
    ns = len(ls)
    cls_count = [0] * 6
    for a in range(ns):
        for b in range(a + 1):
            l1, l2 = max(ls[a], ls[b]), min(ls[a], ls[b])
            cls_count[l1 * (l1 + 1) // 2 + l2] += 1
    npairs = ns * (ns + 1) // 2
    assert sum(cls_count) == npairs
    total = 0
    for cp in range(6):
        for cq in range(cp + 1):
            n_p, n_q = cls_count[cp], cls_count[cq]
            nquart = n_p * (n_p + 1) // 2 if cp == cq else n_p * n_q
            total += nquart
            if cp == cq and n_p:
                for q in list(range(min(nquart, 2000))) + list(range(max(0, nquart - 2000), nquart)):
                    ip, iq = _decode_triangle(q)
                    assert 0 <= iq <= ip < n_p
                    assert ip * (ip + 1) // 2 + iq == q
    assert total == npairs * (npairs + 1) // 2
