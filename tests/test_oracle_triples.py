"""The (T) oracle (oracle/ccsd_t_ref.py) and its pin: the reference's recorded
CCSD(T) run on water (6-31G, cc-pVDZ density fitting, RI-RHF, method df,
frozen core; outputs/h2o-ccsd_t-631g-pvdz.out:233, :336, :395 of its
validation suite), rebuilt from the geometry by the oracle's integral, RI-RHF
and CCSD code (tests/golden/make_ccsd_t.py)."""
import numpy as np
import pytest

from conftest import GOLDEN
from mpqc_gb300 import synth
from oracle import ccsd_t_ref as T


@pytest.mark.parametrize("o,v,seed", [(1, 3, 1), (2, 5, 2), (3, 7, 3), (4, 6, 4)])
def test_triplet_batches_equal_the_full_triples(o, v, seed):
    inp = synth.make_inputs(o, v, 12, seed=seed, t1_scale=1e-2)
    args = (inp.t1, inp.t2, inp.Gijab, inp.Gijka, inp.Giabc, inp.eps_o, inp.eps_v)
    full = T.triples_energy(*args)
    # one occupied orbital: E(T) vanishes (both sums are rounding noise)
    assert abs(T.triples_energy_by_triplet(*args) - full) <= 1e-14 * abs(full) + 1e-20


def test_recorded_triples_energy_is_reproduced():
    g = np.load(GOLDEN / "h2o_ccsd_t_631g.npz")
    e_t = T.triples_energy(g["t1"], g["t2"], g["Gijab"], g["Gijka"], g["Giabc"], g["eps_o"], g["eps_v"])
    assert abs(e_t - float(g["ref_e_t"])) < 1e-11          # recorded: -0.000868413807153793
    assert abs(float(g["oracle_e_ccsd"]) - float(g["ref_e_ccsd"])) < 1e-9
    assert abs(float(g["oracle_e_rhf"]) - float(g["ref_e_rhf"])) < 1e-9


def test_ri_rhf_from_the_geometry():
    """The density-fitted integrals from the C restatement (three- and
    two-centre integrals with a unit s function) give the recorded RI-RHF
    energy, and the fixture's MO blocks are their transform."""
    from oracle import molecule as M
    g = np.load(GOLDEN / "h2o_ccsd_t_631g.npz")
    mol = M.Molecule.from_xyz_text(str(g["xyz"]))
    S, H, B = M.df_factors_c(mol, "6-31G", "cc-pVDZ")
    G = np.einsum("kmn,kls->mnls", B, B)
    scf = M.rhf(S, H, G, mol.n_electrons() // 2, mol.nuclear_repulsion())
    assert abs(scf.energy - float(g["ref_e_rhf"])) < 1e-9
    blocks, eo, ev = M.mo_blocks(scf, G, int(g["n_frozen"]))
    assert np.allclose(eo, g["eps_o"], atol=1e-10) and np.allclose(ev, g["eps_v"], atol=1e-10)
    # orbital phases may differ: compare phase-free quantities
    assert np.allclose(np.abs(blocks["Gijab"]), np.abs(g["Gijab"]), atol=1e-9)
