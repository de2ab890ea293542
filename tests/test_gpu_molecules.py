"""The CUDA solver on water, through the C ABI, against the reference's recorded
CCSD energies and the oracle's amplitudes.

Plain FP64: correlation energy within the recorded run's precision (the rule of
the reference's checker, tests/validation/check.py:81-85 of the MPQC tree) and
within 1e-8 Eh of the oracle, max|dT2| <= 1e-7.  Mixed (split-BF16 bulk
contractions, FP64 refinement): |dE| <= 1e-6 Eh."""
import numpy as np
import pytest

from conftest import freeze_first_occupied, load_molecule, rel_err
from mpqc_gb300 import Solver
from oracle import ccsd_ref as R
from oracle import molecule as M

pytestmark = pytest.mark.gpu

CASES = [("h2o_631g", False), ("h2o_ccpvdz", False), ("h2o_ccpvdz", True)]

# single-water benchmark geometry: O (0, 0, 0.1173), H (0, +-0.7572, -0.4692) Angstrom
WATER_BENCH_XYZ = "3\n\nO 0 0 0.1173\nH 0 0.7572 -0.4692\nH 0 -0.7572 -0.4692\n"


def _case(name, frozen):
    blocks, eo, ev, g = load_molecule(name)
    key = "ref_e_ccsd"
    if frozen:
        blocks, eo = freeze_first_occupied(blocks, eo)
        key = "ref_e_ccsd_fc"
    return blocks, eo, ev, float(g[key]), float(g["precision"]), g


def _solve(blocks, eo, ev, precision="fp64", **kw):
    with Solver(len(eo), len(ev), precision=precision, target_precision=1e-11, max_iter=60, **kw) as s:
        s.set_inputs(eo, ev, **blocks)
        return s.solve()


@pytest.mark.parametrize("name,frozen", CASES)
def test_fp64_solve_reproduces_recorded_energy(name, frozen):
    blocks, eo, ev, e_ref, prec, g = _case(name, frozen)
    e, t1, t2, rep = _solve(blocks, eo, ev)
    assert rep.converged and rep.mixed_iters == 0
    assert abs(e - e_ref) <= prec
    ora = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=1e-11, max_iter=60)
    assert rep.iters == ora.iters
    assert abs(e - ora.e_corr) < 1e-10
    assert np.max(np.abs(t2 - ora.t2)) < 1e-7 and np.max(np.abs(t1 - ora.t1)) < 1e-7


@pytest.mark.parametrize("name,frozen", CASES)
def test_mixed_solve_within_micro_hartree(name, frozen):
    blocks, eo, ev, e_ref, prec, g = _case(name, frozen)
    e, t1, t2, rep = _solve(blocks, eo, ev, precision="mixed", refine_iters=2)
    assert rep.converged and rep.fp64_iters >= 2
    assert abs(e - e_ref) <= 1e-6


@pytest.mark.parametrize("name", ["h2o_631g", "h2o_ccpvdz"])
def test_residual_at_converged_amplitudes(name):
    blocks, eo, ev, g = load_molecule(name)
    t1, t2 = g["t1"], g["t2"]
    r1_ref, r2_ref = R.residual(t1, t2, R.Integrals(**blocks))
    with Solver(len(eo), len(ev)) as s:
        s.set_inputs(eo, ev, **blocks)
        r1, r2 = s.residual(t1, t2)
        e, err = s.energy(t1, t2, r1, r2)
    # converged amplitudes: residuals are at the 1e-11 level, compare absolutely
    assert np.max(np.abs(r2 - r2_ref)) < 1e-13 and np.max(np.abs(r1 - r1_ref)) < 1e-13
    assert abs(e - float(g["oracle_e_ccsd"])) < 1e-10 and err < 1e-10


def test_water_benchmark_geometry_against_oracle():
    """cc-pVDZ water at the single-water benchmark geometry, no frozen core (o=5, v=19):
    converge to 1e-10 and compare E_corr and T2 with the oracle."""
    scf, blocks, eo, ev, nfz = M.molecular_inputs(WATER_BENCH_XYZ, "cc-pVDZ", frozen_core=False)
    assert (len(eo), len(ev), scf.C.shape[0]) == (5, 19, 24)
    ora = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=1e-10, max_iter=60)
    with Solver(5, 19, target_precision=1e-10, max_iter=60) as s:
        s.set_inputs(eo, ev, **{k: np.ascontiguousarray(v) for k, v in blocks.items()})
        e, t1, t2, rep = s.solve()
    assert rep.converged and ora.converged
    assert abs(e - ora.e_corr) < 1e-8
    assert np.max(np.abs(t2 - ora.t2)) < 1e-7
    assert rel_err(t2, ora.t2) < 1e-6
