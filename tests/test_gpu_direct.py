"""The integral-direct residual (method "direct": the U intermediate in the AO
basis, ccsd.h:581-603, ccsd_r1_r2.h:116-118, 282-286) on the GPU, through the
C ABI, against the oracle's restatement of those branches and the reference's
recorded water energies.

Inputs come from the oracle's molecular chain (C restatement of the AO
integrals, RHF, MO blocks): the handle gets (pq|rs) and the MO coefficients
instead of (ab|cd)."""
import numpy as np
import pytest

from conftest import load_molecule, rel_err
from mpqc_gb300 import Solver, _lib, molecules
from oracle import ccsd_ref as R
from oracle import molecule as M

pytestmark = pytest.mark.gpu

MO = ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc")


def _parse_xyz(text):
    rows = [ln.split() for ln in text.strip().splitlines()]
    n = int(rows[0][0])
    body = [r for r in rows[1:] if len(r) >= 4][:n]
    return [r[0] for r in body], np.array([[float(x) for x in r[1:4]] for r in body])


def chain(symbols, coords_angstrom, basis, frozen_core=False):
    mol = M.Molecule(list(symbols), molecules.to_bohr(coords_angstrom))
    S, H, G = M.ao_integrals_c(mol, basis)
    nocc = mol.n_electrons() // 2
    scf = M.rhf(S, H, G, nocc, mol.nuclear_repulsion())
    nfz = mol.n_frozen_core() if frozen_core else 0
    blocks, eo, ev = M.mo_blocks(scf, G, nfz)
    Ci = np.ascontiguousarray(scf.C[:, nfz:nocc])
    Ca = np.ascontiguousarray(scf.C[:, nocc:])
    return G, Ca, Ci, blocks, eo, ev


def _direct_solver(G, Ca, Ci, blocks, eo, ev, **kw):
    s = Solver(len(eo), len(ev), **kw)
    s.set_direct_inputs(eo, ev, G, Ca, Ci, **{k: np.ascontiguousarray(blocks[k]) for k in MO})
    return s


@pytest.fixture(scope="module")
def water():
    sym, xyz = molecules.water()
    return chain(sym, xyz, "cc-pVDZ")


@pytest.mark.parametrize("precision,slices,tol", [("fp64", 3, 1e-12), ("mixed", 3, 2e-6), ("mixed", 2, 2e-5)])
def test_direct_residual_matches_oracle(water, precision, slices, tol):
    G, Ca, Ci, blocks, eo, ev = water
    o, v = len(eo), len(ev)
    rng = np.random.default_rng(3)
    t2 = rng.normal(0.0, 1e-2, (v, v, o, o))
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    t1 = rng.normal(0.0, 1e-2, (v, o))
    ints = R.Integrals(**blocks, Ci=Ci, Ca=Ca)
    r1_ref, r2_ref = R.residual(t1, t2, ints, G_ao=G)
    s1, s2 = R.residual(t1, t2, R.Integrals(**blocks))
    assert rel_err(r2_ref, s2) < 1e-13  # the direct branches equal the standard residual
    with _direct_solver(G, Ca, Ci, blocks, eo, ev, precision=precision, slices=(slices,) * 3) as s:
        r1, r2 = s.residual(t1, t2)
    assert rel_err(r2, r2_ref) < tol and rel_err(r1, r1_ref) < tol


@pytest.mark.parametrize("name,frozen,key", [("h2o_631g", True, "ref_e_ccsd"), ("h2o_ccpvdz", False, "ref_e_ccsd")])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_direct_solve_reproduces_recorded_energy(name, frozen, key, precision):
    """The reference records its water/6-31G CCSD run with method "direct"
    (h2o-ccsd-direct-631g.out:304); the integral-direct path reproduces it."""
    _, _, _, g = load_molecule(name)
    sym, xyz = _parse_xyz(str(g["xyz"]))
    G, Ca, Ci, blocks, eo, ev = chain(sym, xyz, str(g["basis"]), frozen_core=frozen)
    with _direct_solver(G, Ca, Ci, blocks, eo, ev, precision=precision, target_precision=1e-11,
                        max_iter=60) as s:
        e, t1, t2, rep = s.solve()
    assert rep.converged
    tol = float(g["precision"]) if precision == "fp64" else 1e-6
    assert abs(e - float(g[key])) <= tol


def test_direct_handle_kind_is_fixed():
    sym, xyz = molecules.water()
    G, Ca, Ci, blocks, eo, ev = chain(sym, xyz, "6-31G")
    with _direct_solver(G, Ca, Ci, blocks, eo, ev) as s:
        with pytest.raises(_lib.GbccError) as ex:
            s.set_inputs(eo, ev, **{k: np.ascontiguousarray(blocks[k]) for k in MO + ("Gabcd",)})
        assert ex.value.status == _lib.GBCC_ERR_STATE
