"""(T) on the GPU (gbcc_triples) against the oracle's restatement of the
reference's straight (T) and against the reference's recorded CCSD(T) water
energies (tests/golden/h2o_ccsd_t_631g.npz)."""
import numpy as np
import pytest

from conftest import GOLDEN, ints_dict
from mpqc_gb300 import Solver, _lib, synth
from oracle import ccsd_t_ref as T

pytestmark = pytest.mark.gpu

# |dE(T)| / |E(T)|: FP64 and FP64_TC at the level of FP64 sums, mixed at the
# three-slice contraction error
TOL = {"fp64": 1e-12, "fp64_tc": 1e-11, "mixed": 2e-5}


def _solver(inp, **kw):
    s = Solver(inp.o, inp.v, **kw)
    s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
    return s


@pytest.mark.parametrize("precision", ["fp64", "fp64_tc", "mixed"])
@pytest.mark.parametrize("o,v,seed", [(1, 3, 1), (3, 7, 2), (5, 19, 3), (7, 33, 4), (10, 40, 5)])
def test_triples_match_the_oracle(o, v, seed, precision):
    inp = synth.make_inputs(o, v, 16, seed=seed, t1_scale=1e-2)
    ref = T.triples_energy_by_triplet(inp.t1, inp.t2, inp.Gijab, inp.Gijka, inp.Giabc, inp.eps_o, inp.eps_v)
    with _solver(inp, precision="fp64_tc" if precision == "fp64_tc" else "fp64") as s:
        e = s.triples(precision, inp.t1, inp.t2)
    print(f"o={o} v={v} {precision}: E(T) {e:.15e} oracle {ref:.15e} rel {abs(e - ref) / abs(ref):.2e}")
    # o = 1: E(T) is zero by exact cancellation, which split precision leaves at ~1e-14
    assert abs(e - ref) <= TOL[precision] * abs(ref) + (1e-12 if precision == "mixed" else 1e-16)


@pytest.fixture(scope="module")
def water_t():
    g = np.load(GOLDEN / "h2o_ccsd_t_631g.npz")
    blocks = {k: np.ascontiguousarray(g[k]) for k in
              ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc", "Gabcd")}
    return g, blocks


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp64_tc", 1e-11), ("mixed", 1e-8)])
def test_recorded_ccsd_t_from_the_solve(water_t, precision, tol):
    """CCSD then (T) on the reference's DF water inputs: the recorded CCSD
    (stopped at dE 2.6e-10) and (T) energies."""
    g, blocks = water_t
    eo, ev = g["eps_o"], g["eps_v"]
    with Solver(eo.size, ev.size, precision="fp64", target_precision=1e-11, max_iter=60) as s:
        s.set_inputs(eo, ev, **blocks)
        e, _, _, rep = s.solve(want_amplitudes=False)
        assert rep.converged and abs(e - float(g["ref_e_ccsd"])) < 1e-9
        e_t = s.triples(precision)
    assert abs(e_t - float(g["ref_e_t"])) < tol


def test_recorded_triples_through_the_df_inputs(water_t):
    """The same run through the density-fitted inputs (the reference's
    method df: (ab|cd) never formed, <ia|bc> built from the factors)."""
    g, blocks = water_t
    eo, ev = g["eps_o"], g["eps_v"]
    names = ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka")
    with Solver(eo.size, ev.size, precision="fp64", target_precision=1e-11, max_iter=60) as s:
        s.set_df_inputs(eo, ev, np.ascontiguousarray(g["Xai"]), np.ascontiguousarray(g["Xab"]),
                        **{k: blocks[k] for k in names})
        e, _, _, rep = s.solve(want_amplitudes=False)
        e_t = s.triples("fp64")
    assert rep.converged and abs(e - float(g["ref_e_ccsd"])) < 1e-9
    assert abs(e_t - float(g["ref_e_t"])) < 1e-11


def test_triples_argument_errors():
    inp = synth.make_inputs(2, 5, 8, seed=9, t1_scale=1e-2)
    with _solver(inp) as s:
        with pytest.raises(_lib.GbccError) as ex:
            s.triples("fp64")                       # no solve, no amplitudes
        assert ex.value.status == _lib.GBCC_ERR_STATE
        with pytest.raises(_lib.GbccError) as ex:
            s.triples("fp64", inp.t1, None)
        assert ex.value.status == _lib.GBCC_ERR_INVALID_ARG
        bad = inp.t2.copy()
        bad[0, 1, 0, 1] += 1e-3                     # not pair-symmetric
        with pytest.raises(_lib.GbccError) as ex:
            s.triples("fp64", inp.t1, bad)
        assert ex.value.status == _lib.GBCC_ERR_INVALID_ARG


def test_keyval_ccsd_t_front_end(water_t):
    """The KeyVal front end (CCSD(T), method df, approach straight as in the
    recorded input) gives the recorded CCSD(T) energy."""
    from mpqc_gb300 import CCSD_T
    g, blocks = water_t
    ints = {k: blocks[k] for k in ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka")}
    ints.update(Xai=np.ascontiguousarray(g["Xai"]), Xab=np.ascontiguousarray(g["Xab"]))
    w = CCSD_T({"ref": "scf", "method": "df", "approach": "straight", "precision": 1e-11, "max_iter": 60})
    e = w.compute(g["eps_o"], g["eps_v"], ints)
    assert abs(w.triples_energy - float(g["ref_e_t"])) < 1e-11
    assert abs(e - float(g["ref_e_ccsd"]) - float(g["ref_e_t"])) < 1e-9


@pytest.mark.parametrize("chunk", [1, 2, 4])
def test_triplet_chunks_give_the_same_energy(chunk):
    """Batches of `chunk` triplets (the size large v takes to keep each t3 slice
    in L2) give the energy of whole batches."""
    from mpqc_gb300 import _lib as L
    lib = L.load()
    inp = synth.make_inputs(5, 19, 16, seed=3, t1_scale=1e-2)
    ref = T.triples_energy_by_triplet(inp.t1, inp.t2, inp.Gijab, inp.Gijka, inp.Giabc, inp.eps_o, inp.eps_v)
    try:
        assert lib.gbcc_testing_triples_chunk(chunk) == 0
        with _solver(inp) as s:
            e = {p: s.triples(p, inp.t1, inp.t2) for p in ("fp64", "mixed")}
    finally:
        lib.gbcc_testing_triples_chunk(0)
    assert abs(e["fp64"] - ref) <= 1e-12 * abs(ref)
    assert abs(e["mixed"] - ref) <= 2e-5 * abs(ref)
