"""CPU checks of the density-fitted oracle (oracle/ccsd_df_ref.py).

With every four-index block built from one factor, <pq|rs> = sum_K B[K,p,r]
B[K,q,s], the density-fitted residual (three-index factors in the Fock-like
intermediates, the ring's Gijab T term and the lazy ladder with the T1 terms
folded into a modified factor) is an exact rearrangement of the standard
residual, so the two oracles agree to rounding.  This pins the restatement
without running the reference."""
import numpy as np
import pytest

from conftest import oracle_ints, rel_err
from mpqc_gb300 import synth
from oracle import ccsd_df_ref as D
from oracle import ccsd_ref as R


def df_case(o, v, naux, seed, t1_scale):
    rng = np.random.default_rng(seed)
    B = synth.make_df_factor(rng, naux, o + v, 0.05)
    eps_o = np.sort(rng.uniform(-1.5, -0.3, size=o))
    eps_v = np.sort(rng.uniform(0.1, 3.0, size=v))
    t2 = rng.normal(0.0, 1e-2, size=(v, v, o, o))
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    t1 = rng.normal(0.0, t1_scale, size=(v, o))
    return B, synth.inputs_from_factor(B, eps_o, eps_v, t1, t2)


@pytest.mark.parametrize("o,v,naux,seed,t1_scale", [(3, 7, 20, 1, 1e-2), (5, 11, 40, 2, 3e-2), (4, 9, 30, 3, 0.0)])
def test_df_residual_equals_standard_residual(o, v, naux, seed, t1_scale):
    B, inp = df_case(o, v, naux, seed, t1_scale)
    r1, r2 = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    d1, d2 = D.residual_df(inp.t1, inp.t2, oracle_ints(inp), *D.df_factors(B, o))
    assert rel_err(d1, r1) < 1e-12
    assert rel_err(d2, r2) < 1e-12


def test_df_residual_keeps_pair_symmetry_and_sets_fock_intermediates():
    B, inp = df_case(4, 10, 30, 7, 2e-2)
    ints = oracle_ints(inp)
    _, d2 = D.residual_df(inp.t1, inp.t2, ints, *D.df_factors(B, 4))
    assert np.max(np.abs(d2 - d2.transpose(1, 0, 3, 2))) < 1e-14 * np.max(np.abs(d2))
    std = oracle_ints(inp)
    R.residual(inp.t1, inp.t2, std)
    assert rel_err(ints.FAB, std.FAB) < 1e-12 and rel_err(ints.FIJ, std.FIJ) < 1e-12
