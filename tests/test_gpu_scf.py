"""The GPU input producer (AO integrals, RHF, AO -> MO transform into the CCSD
handle) against the oracle's integrals and the reference's recorded energies.

* AO integrals of a water dimer (cc-pVDZ, 48 functions, every shell-quartet
  class up to (dd|dd)) and water (6-31G) against the C restatement of the
  oracle: S and H within 1e-12, (mu nu|la si) within 1e-12 absolute.
* RHF energies of the reference's water within 1e-9 Eh of its recorded ones
  (outputs h2o-ccsd-direct-631g.out:228, h2o-eom-ip-ccsd-pvdz.out:219).
* Geometry -> RHF -> CCSD entirely on the GPU reproduces the recorded CCSD
  energies within each run's precision (the reference checker's rule).
* Water dimer geometry -> CCSD on the GPU against the oracle's whole chain
  (C integrals, numpy RHF and transform, numpy CCSD): |dE| < 1e-9 Eh in FP64,
  <= 1e-6 Eh mixed.
"""
import numpy as np
import pytest

from conftest import load_molecule

pytestmark = pytest.mark.gpu


def _parse_xyz(text):
    rows = [ln.split() for ln in text.strip().splitlines()]
    n = int(rows[0][0])
    body = [r for r in rows[1:] if len(r) >= 4][:n]
    return [r[0] for r in body], np.array([[float(x) for x in r[1:4]] for r in body])


def _oracle_ao(symbols, coords_angstrom, basis):
    from mpqc_gb300 import molecules
    from oracle import molecule as M
    mol = M.Molecule(list(symbols), molecules.to_bohr(coords_angstrom))
    return mol, M.ao_integrals_c(mol, basis)


@pytest.mark.parametrize("system,basis", [("dimer", "cc-pVDZ"), ("water", "6-31G"), ("water", "cc-pVDZ")])
def test_ao_integrals_match_oracle(system, basis):
    from mpqc_gb300 import RHF, molecules
    sym, xyz = molecules.water_cluster(2, seed=5) if system == "dimer" else molecules.water()
    _, (S0, H0, G0) = _oracle_ao(sym, xyz, basis)
    with RHF(sym, xyz, basis) as scf:
        S, H, G = scf.ao(eri=True)
    assert S.shape == S0.shape and G.shape == G0.shape
    assert np.max(np.abs(S - S0)) < 1e-12
    assert np.max(np.abs(H - H0)) < 1e-11
    assert np.max(np.abs(G - G0)) < 1e-12
    # the eight-fold permutational symmetry of what was written (to rounding:
    # a shell paired with itself computes (mu nu| and (nu mu| separately)
    scale = np.max(np.abs(G))
    assert np.max(np.abs(G - G.transpose(1, 0, 2, 3))) < 1e-15 * scale
    assert np.max(np.abs(G - G.transpose(2, 3, 0, 1))) < 1e-15 * scale


@pytest.mark.parametrize("name", ["h2o_631g", "h2o_ccpvdz"])
def test_rhf_reproduces_recorded_energy(name):
    from mpqc_gb300 import RHF
    _, _, _, g = load_molecule(name)
    sym, xyz = _parse_xyz(str(g["xyz"]))
    with RHF(sym, xyz, str(g["basis"]), threshold=1e-12, max_iter=60) as scf:
        e = scf.run()
        assert scf.report.converged
    assert abs(e - float(g["ref_e_rhf"])) < 1e-9
    assert abs(e - float(g["oracle_e_rhf"])) < 1e-9


@pytest.mark.parametrize("name,frozen,key", [("h2o_631g", True, "ref_e_ccsd"), ("h2o_ccpvdz", False, "ref_e_ccsd"),
                                             ("h2o_ccpvdz", True, "ref_e_ccsd_fc")])
def test_geometry_to_ccsd_on_gpu_reproduces_recorded_energy(name, frozen, key):
    from mpqc_gb300 import ccsd_energy
    _, _, _, g = load_molecule(name)
    sym, xyz = _parse_xyz(str(g["xyz"]))
    e_scf, e, rep, srep = ccsd_energy(sym, xyz, str(g["basis"]), frozen_core=frozen, precision="fp64",
                                      target_precision=1e-11, max_iter=60, scf_threshold=1e-12)
    assert rep.converged and srep.converged
    assert abs(e_scf - float(g["ref_e_rhf"])) < 1e-9
    assert abs(e - float(g[key])) <= float(g["precision"])


@pytest.fixture(scope="module")
def dimer_oracle():
    from mpqc_gb300 import molecules
    from oracle import ccsd_ref as R
    from oracle import molecule as M
    sym, xyz = molecules.water_cluster(2, seed=5)
    mol, (S, H, G) = _oracle_ao(sym, xyz, "cc-pVDZ")
    scf = M.rhf(S, H, G, mol.n_electrons() // 2, mol.nuclear_repulsion())
    blocks, eo, ev = M.mo_blocks(scf, G, 0)
    ora = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=1e-10, max_iter=60)
    assert ora.converged
    return sym, xyz, scf.energy, ora.e_corr


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_water_dimer_geometry_to_ccsd_matches_oracle(dimer_oracle, precision):
    from mpqc_gb300 import ccsd_energy
    sym, xyz, e_rhf, e_corr = dimer_oracle
    e_scf, e, rep, srep = ccsd_energy(sym, xyz, "cc-pVDZ", precision=precision, target_precision=1e-10,
                                      max_iter=60, scf_threshold=1e-12)
    assert srep.nbf == 48 and srep.nocc == 10
    assert abs(e_scf - e_rhf) < 1e-9
    assert rep.converged
    assert abs(e - e_corr) < (1e-9 if precision == "fp64" else 1e-6)


def test_ccsd_inputs_reject_mismatched_handle():
    from mpqc_gb300 import RHF, Solver, _lib as L, molecules
    sym, xyz = molecules.water()
    with RHF(sym, xyz, "cc-pVDZ") as scf:
        with pytest.raises(L.GbccError) as ex:
            with Solver(5, 19) as s:
                scf.ccsd_inputs(s)  # before the SCF has run
        assert ex.value.status == L.GBCC_ERR_STATE
        scf.run()
        with pytest.raises(L.GbccError) as ex:
            with Solver(4, 19) as s:
                scf.ccsd_inputs(s)  # o does not match
        assert ex.value.status == L.GBCC_ERR_INVALID_ARG
