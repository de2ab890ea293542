"""Many independent molecules solved at once (gbcc_solve_batch): each handle's
solve runs on its own stream from its own host thread.  The batch has no
counterpart in the reference (one molecule per run); its results must equal
the same handles solved one after another, and the polarised Pople basis it is
exercised with (Cartesian d shells) is checked against the oracle's chain."""
import numpy as np
import pytest

from mpqc_gb300 import RHF, Solver, _lib, molecules, solve_batch

pytestmark = pytest.mark.gpu


def _handles(specs, basis, precision, **kw):
    out = []
    for n, seed in specs:
        sym, xyz = molecules.water_cluster(n, seed=seed)
        with RHF(sym, xyz, basis, threshold=1e-11, max_iter=60) as scf:
            scf.run()
            o = scf.nocc()
            s = Solver(o, scf.nbf - o, precision=precision, max_iter=60, autotune=False, **kw)
            scf.ccsd_inputs(s)
            out.append(s)
    return out


SPECS = [(1, 11), (2, 12), (1, 13), (3, 14), (2, 15)]


@pytest.mark.parametrize("precision,target", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_batch_equals_one_by_one(precision, target):
    hs = _handles(SPECS, "6-31G*", precision, target_precision=target)
    try:
        alone = [s.solve(want_amplitudes=False) for s in hs]
        batch = solve_batch(hs)
        again = solve_batch(hs)  # repeated batches restart from t = 0 and agree
        for (e, _, _, r), (eb, rb), (ea, _) in zip(alone, batch, again):
            assert r.converged and rb.converged
            assert rb.iters == r.iters
            assert abs(eb - e) <= 1e-12 * abs(e)
            assert ea == eb
    finally:
        for s in hs:
            s.close()


def test_batch_fp64_matches_the_oracle_chain():
    from oracle import ccsd_ref as R
    from oracle import molecule as M
    specs = [(1, 21), (2, 22)]
    hs = _handles(specs, "6-31G*", "fp64", target_precision=1e-11)
    try:
        got = solve_batch(hs)
    finally:
        for s in hs:
            s.close()
    for (n, seed), (e, rep) in zip(specs, got):
        sym, xyz = molecules.water_cluster(n, seed=seed)
        mol = M.Molecule(list(sym), molecules.to_bohr(xyz))
        S, H, G = M.ao_integrals_c(mol, "6-31G*")
        scf = M.rhf(S, H, G, mol.n_electrons() // 2, mol.nuclear_repulsion())
        blocks, eo, ev = M.mo_blocks(scf, G, 0)
        ora = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=1e-11, max_iter=60)
        assert rep.converged and ora.converged
        assert abs(e - ora.e_corr) < 1e-9


def test_batch_argument_errors():
    hs = _handles([(1, 31)], "6-31G", "fp64")
    s = hs[0]
    try:
        with pytest.raises(_lib.GbccError) as ex:
            solve_batch([s, s])
        assert ex.value.status == _lib.GBCC_ERR_INVALID_ARG
        assert solve_batch([]) == []
        # a handle without inputs fails its solve; the batch reports it and
        # the other handle still completes
        empty = Solver(s.o, s.v)
        try:
            with pytest.raises(_lib.GbccError) as ex:
                solve_batch([s, empty])
            assert ex.value.status == _lib.GBCC_ERR_STATE
            e, _, _, r = s.solve(want_amplitudes=False)
            assert r.converged and e < 0
        finally:
            empty.close()
    finally:
        s.close()
