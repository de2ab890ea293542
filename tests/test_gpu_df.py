"""The density-fitted residual (method "df", lazy (ab|cd) ladder) on the GPU
against the oracle's restatement of compute_cs_ccsd_r1_df / r2_df
(oracle/ccsd_df_ref.py), through the C ABI.

The handle gets three-index factors instead of Giabc and Gabcd; the ladder
builds G+- rows one block of a at a time from the factors.  FP64 residuals
agree with the oracle to 1e-12 of max|r|, split-BF16 ones within the bars of
the standard path, with one block and with several (a block size forced by the
test hook), and a DF solve reaches the oracle's energy."""
import numpy as np
import pytest

from conftest import rel_err
from mpqc_gb300 import Solver, _lib, synth
from oracle import ccsd_df_ref as D
from oracle import ccsd_ref as R

pytestmark = pytest.mark.gpu

FOUR = ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka")


def df_case(o, v, naux, seed, t1_scale=1e-2):
    rng = np.random.default_rng(seed)
    B = synth.make_df_factor(rng, naux, o + v, 0.05)
    eps_o = np.sort(rng.uniform(-1.5, -0.3, size=o))
    eps_v = np.sort(rng.uniform(0.1, 3.0, size=v))
    t2 = rng.normal(0.0, 1e-2, size=(v, v, o, o))
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    t1 = rng.normal(0.0, t1_scale, size=(v, o))
    inp = synth.inputs_from_factor(B, eps_o, eps_v, t1, t2)
    Xai, Xab, Xij = D.df_factors(B, o)
    return inp, Xai, Xab, Xij


def _df_solver(inp, Xai, Xab, block_rows=0, **kw):
    lib = _lib.load()
    assert lib.gbcc_testing_df_block_rows(block_rows) == 0
    try:
        s = Solver(inp.o, inp.v, **kw)
        s.set_df_inputs(inp.eps_o, inp.eps_v, Xai, Xab,
                        **{k: np.ascontiguousarray(getattr(inp, k)) for k in FOUR})
    finally:
        lib.gbcc_testing_df_block_rows(0)
    return s


@pytest.mark.parametrize("o,v,naux,blk", [(3, 7, 20, 0), (5, 19, 30, 0), (6, 30, 40, 7), (8, 40, 30, 3)])
@pytest.mark.parametrize("precision,slices,tol", [("fp64", 3, 1e-12), ("mixed", 3, 2e-6), ("mixed", 2, 2e-5)])
def test_df_residual_matches_oracle(o, v, naux, blk, precision, slices, tol):
    inp, Xai, Xab, Xij = df_case(o, v, naux, seed=o * 7 + v)
    ints = R.Integrals(**{k: getattr(inp, k) for k in FOUR}, Giabc=None, Gabcd=None)
    r1_ref, r2_ref = D.residual_df(inp.t1, inp.t2, ints, Xai, Xab, Xij)
    with _df_solver(inp, Xai, Xab, blk, precision=precision, slices=(slices,) * 3) as s:
        r1, r2 = s.residual(inp.t1, inp.t2)
    assert rel_err(r2, r2_ref) < tol and rel_err(r1, r1_ref) < tol


def test_df_and_standard_handles_agree():
    inp, Xai, Xab, _ = df_case(6, 24, 30, seed=5)
    with _df_solver(inp, Xai, Xab, 5) as s:
        d1, d2 = s.residual(inp.t1, inp.t2)
    with Solver(6, 24) as s:
        s.set_inputs(inp.eps_o, inp.eps_v, **{k: np.ascontiguousarray(getattr(inp, k)) for k in
                                              FOUR + ("Giabc", "Gabcd")})
        f1, f2 = s.residual(inp.t1, inp.t2)
    assert rel_err(d2, f2) < 1e-12 and rel_err(d1, f1) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_df_solve_reaches_the_oracle_energy(precision):
    inp, Xai, Xab, _ = df_case(5, 19, 30, seed=22, t1_scale=0.0)
    ints = R.Integrals(**{k: getattr(inp, k) for k in FOUR + ("Giabc", "Gabcd")})
    ref = R.solve_ccsd(ints, inp.eps_o, inp.eps_v, target_precision=1e-10, max_iter=60)
    with _df_solver(inp, Xai, Xab, 4, precision=precision, target_precision=1e-10, max_iter=60) as s:
        e, t1, t2, rep = s.solve()
    assert rep.converged
    assert abs(e - ref.e_corr) < (1e-10 if precision == "fp64" else 1e-6)
    if precision == "fp64":
        assert rep.iters == ref.iters and np.max(np.abs(t2 - ref.t2)) < 1e-8


def test_handle_kind_is_fixed_by_the_first_inputs():
    inp, Xai, Xab, _ = df_case(3, 7, 20, seed=1)
    with _df_solver(inp, Xai, Xab) as s:
        with pytest.raises(_lib.GbccError) as ex:
            s.set_inputs(inp.eps_o, inp.eps_v, **{k: np.ascontiguousarray(getattr(inp, k)) for k in
                                                  FOUR + ("Giabc", "Gabcd")})
        assert ex.value.status == _lib.GBCC_ERR_STATE
