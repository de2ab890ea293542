"""Parity of the CUDA residual engine and solver with the FP64 oracle,
called through the C ABI (mpqc_gb300.Solver -> libgbcc)."""
import numpy as np
import pytest

from conftest import ints_dict, load_golden, oracle_ints, rel_err
from mpqc_gb300 import Solver, synth
from mpqc_gb300 import _lib as L
from mpqc_gb300._lib import GbccError
from oracle import ccsd_ref as R

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12          # max|dr| / max|r_ref|, plain FP64 path
# split-BF16 path, max|dr| / max|r_ref| by slice count: about 4x the largest
# error measured against the oracle (3 slices 5.1e-7, 2 slices 5.3e-6, 1 slice
# 2.5e-3, at sizes up to o = 32, v = 160)
MIXED_TOL = {3: 2e-6, 2: 2e-5, 1: 1e-2}


def _solver(inp, precision="fp64", slices=(3, 3, 3), **kw):
    s = Solver(inp.o, inp.v, precision=precision, slices=slices, **kw)
    s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
    return s


@pytest.mark.parametrize("name", ["residual_o3_v7", "residual_o5_v19"])
def test_residual_fp64_golden(name):
    inp, g = load_golden(name)
    with _solver(inp) as s:
        r1, r2 = s.residual(g["t1"], g["t2"])
    assert rel_err(r1, g["r1"]) < FP64_TOL
    assert rel_err(r2, g["r2"]) < FP64_TOL


@pytest.mark.parametrize("o,v,naux", [(1, 1, 3), (1, 2, 4), (2, 3, 5), (4, 9, 12), (3, 33, 20),
                                      (7, 12, 16), (8, 40, 30)])
def test_residual_fp64_random(o, v, naux):
    inp = synth.make_inputs(o, v, naux, seed=o * 100 + v, t1_scale=1e-2)
    r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    with _solver(inp) as s:
        r1, r2 = s.residual(inp.t1, inp.t2)
    assert rel_err(r1, r1_ref) < FP64_TOL
    assert rel_err(r2, r2_ref) < FP64_TOL
    assert np.allclose(r2, r2.transpose(1, 0, 3, 2), rtol=0, atol=1e-14 * np.max(np.abs(r2)))


@pytest.mark.parametrize("slices", [3, 2, 1])
@pytest.mark.parametrize("o,v,naux", [(4, 9, 12), (8, 40, 30), (12, 70, 60), (16, 72, 40), (32, 40, 30),
                                      (40, 48, 30)])
def test_residual_mixed(o, v, naux, slices):
    """(16, 72): the short (K = o) contractions into o^2 v^2 outputs run on the
    CUDA-core stream kernel; (32, 40): also the one with N = o = 32, its t2
    operand read in place; (40, 48): K = o = 40 (the kernel's 64-wide form).
    Every size runs the tensor-core contractions."""
    inp = synth.make_inputs(o, v, naux, seed=o * 10 + v, t1_scale=1e-2)
    r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    with _solver(inp, precision="mixed", slices=(slices,) * 3) as s:
        r1, r2 = s.residual(inp.t1, inp.t2)
        f1, f2 = s.residual(inp.t1, inp.t2, precision="fp64")
    print(f"o={o} v={v} slices={slices}: r2 {rel_err(r2, r2_ref):.2e}, r1 {rel_err(r1, r1_ref):.2e}")
    assert rel_err(r2, r2_ref) < MIXED_TOL[slices]
    assert rel_err(r1, r1_ref) < MIXED_TOL[slices]
    assert rel_err(f2, r2_ref) < FP64_TOL


@pytest.fixture(scope="module")
def production_case():
    """o = 32, v = 160 with FP64 DF integrals (naux 300), t1 != 0: the ladder
    contracts over v (v + 1) / 2 = 12880 pair columns, the ring terms over
    o v = 5120, long enough for the chunked TMEM accumulation and the
    float-float folding to matter.  The oracle residual takes ~20 s on the host."""
    inp = synth.make_inputs(32, 160, 300, seed=61, t1_scale=1e-3, b_scale=0.03)
    r1, r2 = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    return inp, r1, r2


@pytest.mark.parametrize("precision,slices,tol", [("fp64", 3, FP64_TOL), ("mixed", 3, 2e-6), ("mixed", 2, 2e-5)])
def test_residual_at_production_contraction_lengths(production_case, precision, slices, tol):
    inp, r1_ref, r2_ref = production_case
    with _solver(inp, precision=precision, slices=(slices,) * 3) as s:
        r1, r2 = s.residual(inp.t1, inp.t2)
    e2, e1 = rel_err(r2, r2_ref), rel_err(r1, r1_ref)
    print(f"o=32 v=160 {precision} slices={slices}: r2 {e2:.2e}, r1 {e1:.2e}")
    assert e2 < tol and e1 < tol


def test_residual_repeat_identical():
    inp = synth.make_inputs(5, 20, 16, seed=3, t1_scale=1e-2)
    with _solver(inp, precision="mixed") as s:
        a = s.residual(inp.t1, inp.t2)
        b = s.residual(inp.t1, inp.t2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_energy_matches_oracle():
    inp = synth.make_inputs(4, 11, 12, seed=9, t1_scale=1e-2)
    r1, r2 = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    with _solver(inp) as s:
        e, err = s.energy(inp.t1, inp.t2, r1, r2)
    tau = R.make_tau(inp.t1, inp.t2)
    g = inp.Gijab.transpose(2, 3, 0, 1)
    e_ref = 2 * np.vdot(inp.Fia.T + r1, inp.t1) + np.vdot(g + r2, 2 * tau - tau.transpose(1, 0, 2, 3))
    assert abs(e - e_ref) < 1e-13 * max(1.0, abs(e_ref))
    assert abs(err - R.solver_error(r1, r2)) < 1e-15 + 1e-12 * err


def test_solve_fp64_golden():
    inp, g = load_golden("solve_o3_v8")
    with _solver(inp, target_precision=1e-11, max_iter=60) as s:
        e, t1, t2, rep = s.solve()
    assert rep.converged and rep.iters == int(g["iters"])
    assert abs(e - float(g["e_corr"])) < 1e-10
    assert np.max(np.abs(t2 - g["t2"])) < 1e-9
    assert np.max(np.abs(t1 - g["t1"])) < 1e-9


@pytest.mark.parametrize("o,v,naux,seed", [(3, 10, 14, 21), (5, 19, 30, 22), (6, 30, 40, 23)])
def test_solve_fp64_random(o, v, naux, seed):
    inp = synth.make_inputs(o, v, naux, seed=seed, b_scale=0.03)
    ref = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, target_precision=1e-10, max_iter=60)
    with _solver(inp, target_precision=1e-10, max_iter=60) as s:
        e, t1, t2, rep = s.solve()
    assert rep.converged == ref.converged and rep.iters == ref.iters
    assert abs(e - ref.e_corr) < 1e-9
    assert np.max(np.abs(t2 - ref.t2)) < 1e-7


def test_solve_mixed_with_fp64_refinement():
    inp = synth.make_inputs(8, 40, 40, seed=31, b_scale=0.02)
    ref = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, target_precision=1e-10, max_iter=60)
    with _solver(inp, precision="mixed", target_precision=1e-10, max_iter=60, refine_iters=2) as s:
        e, t1, t2, rep = s.solve()
    assert rep.converged and rep.mixed_iters > 0 and rep.fp64_iters >= 2
    assert abs(e - ref.e_corr) < 1e-6
    assert np.max(np.abs(t2 - ref.t2)) < 1e-6


def test_device_pointers_match_host():
    torch = pytest.importorskip("torch")
    inp = synth.make_inputs(4, 13, 12, seed=5, t1_scale=1e-2)
    with _solver(inp) as s:
        h1, h2 = s.residual(inp.t1, inp.t2)
        d1, d2 = s.residual(torch.from_numpy(inp.t1).cuda(), torch.from_numpy(inp.t2).cuda())
    assert np.array_equal(h1, d1.cpu().numpy()) and np.array_equal(h2, d2.cpu().numpy())


def test_zero_copy_inputs_twice_match_host_inputs():
    """gbcc_device_inputs / gbcc_commit_inputs twice on one handle: the commit
    gives the (ab|cd) storage back and the next gbcc_device_inputs takes it
    again, so a refill with other integrals gives that input's residual."""
    torch = pytest.importorskip("torch")

    class _Dev:
        def __init__(self, ptr, shape):
            self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f8", "data": (int(ptr), False),
                                             "version": 3, "strides": None}

    with _solver(synth.make_inputs(4, 13, 12, seed=5, t1_scale=1e-2)) as s:
        for seed in (6, 7):
            inp = synth.make_inputs(4, 13, 12, seed=seed, t1_scale=1e-2)
            ptr = s.device_inputs()
            arrays = dict(ints_dict(inp), eps_o=inp.eps_o, eps_v=inp.eps_v)
            for name, x in arrays.items():
                torch.as_tensor(_Dev(ptr[name], x.shape), device="cuda").copy_(torch.from_numpy(x))
            s.commit_inputs()
            r1, r2 = s.residual(inp.t1, inp.t2)
            r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
            assert rel_err(r2, r2_ref) < FP64_TOL and rel_err(r1, r1_ref) < FP64_TOL


def test_call_order_and_argument_errors():
    inp = synth.make_inputs(2, 5, 6, seed=1)
    s = Solver(2, 5)
    with pytest.raises(GbccError) as e:
        s.residual(inp.t1, inp.t2)
    assert e.value.status == 6  # GBCC_ERR_STATE
    bad = dict(ints_dict(inp))
    eps_o = inp.eps_o.copy()
    eps_o[0] = np.nan
    with pytest.raises(GbccError) as e:
        s.set_inputs(eps_o, inp.eps_v, **bad)
    assert e.value.status == 1  # GBCC_ERR_INVALID_ARG
    s.set_inputs(inp.eps_o, inp.eps_v, **bad)
    r1, r2 = s.residual(inp.t1, inp.t2)
    assert np.all(np.isfinite(r2))
    s.close()


def test_max_iter_reports_not_converged():
    inp = synth.make_inputs(3, 8, 10, seed=2)
    with _solver(inp, max_iter=2) as s:
        e, t1, t2, rep = s.solve()
    assert not rep.converged and rep.iters == 2 and np.isfinite(e)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_matches_direct_launches(precision):
    """The captured residual graph reads the amplitudes of each call: replaying it
    on new t1/t2 gives bitwise the results of direct launches."""
    inp = synth.make_inputs(6, 30, 20, seed=41, t1_scale=1e-2)
    t1b, t2b = inp.t1 * 0.5, inp.t2 * 1.3
    with _solver(inp, precision=precision) as g, _solver(inp, precision=precision, use_graphs=False) as d:
        ga, gb, gc = g.residual(inp.t1, inp.t2), g.residual(t1b, t2b), g.residual(inp.t1, inp.t2)
        da, db = d.residual(inp.t1, inp.t2), d.residual(t1b, t2b)
    for x, y in ((ga, da), (gb, db), (gc, da)):
        assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
    assert not np.array_equal(ga[1], gb[1])


def test_graph_solve_matches_direct_solve():
    inp = synth.make_inputs(5, 24, 20, seed=43, b_scale=0.03)
    with _solver(inp, precision="mixed", target_precision=1e-10, max_iter=60) as g:
        eg, t1g, t2g, rg = g.solve()
    with _solver(inp, precision="mixed", target_precision=1e-10, max_iter=60, use_graphs=False) as d:
        ed, t1d, t2d, rd = d.solve()
    assert rg.iters == rd.iters and eg == ed and np.array_equal(t2g, t2d)


@pytest.mark.parametrize("precision,max_iter", [("fp64", 60), ("mixed", 60), ("mixed", 7), ("fp64", 3)])
def test_whole_solve_graph_makes_the_host_loops_decisions(precision, max_iter):
    """use_graphs = 2 (the loop as one graph, convergence decided on the device)
    gives the host-driven loop's iterations, phase switch, energy and
    amplitudes bit for bit, converged or stopped at max_iter."""
    inp = synth.make_inputs(5, 24, 20, seed=43, b_scale=0.03)
    kw = dict(precision=precision, target_precision=1e-10, max_iter=max_iter)
    if precision == "mixed":
        kw["slices"] = (2, 2, 2)
    runs = []
    for ug in (1, 2):
        with _solver(inp, use_graphs=ug, **kw) as s:
            e, t1, t2, rep = s.solve()
            e2, u1, u2, rep2 = s.solve()   # the graph is replayed
        runs.append((e, t1, t2, rep, e2, u2, rep2))
    (e1, a1, b1, r1, f1, c1, q1), (eg, ag, bg, rg, fg, cg, qg) = runs
    assert (rg.iters, rg.mixed_iters, rg.fp64_iters, rg.converged) == (r1.iters, r1.mixed_iters, r1.fp64_iters,
                                                                     r1.converged)
    assert eg == e1 and np.array_equal(bg, b1) and np.array_equal(ag, a1)
    assert fg == eg and np.array_equal(cg, bg) and qg.iters == rg.iters
    assert rg.converged == (max_iter == 60)
    if precision == "mixed" and max_iter == 60:
        assert rg.mixed_iters > 0 and rg.fp64_iters >= 2 and rg.seconds_residual_mixed > 0.0


def test_whole_solve_graph_restart():
    inp = synth.make_inputs(5, 19, 30, seed=22)
    with _solver(inp, use_graphs=2, target_precision=1e-10, max_iter=40) as s:
        e0, t1, t2, rep0 = s.solve()
        s.set_amplitudes(t1, t2)
        e1, _, u2, rep1 = s.solve()
    assert rep1.converged and rep1.iters <= 2 and abs(e1 - e0) < 1e-10


def test_automatic_slices_follow_measured_error():
    """Slice counts 0 are chosen at set_inputs from the measured residual change
    against 3 slices; the residual stays within the tolerance of the 3-slice one."""
    inp = synth.make_inputs(8, 40, 30, seed=51, t1_scale=1e-2, b_scale=0.03)
    r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    with _solver(inp, precision="mixed", slices=(0, 0, 0)) as s:
        sl, err = s.slice_policy()
        r1, r2 = s.residual(inp.t1, inp.t2)
    with _solver(inp, precision="mixed", slices=(3, 3, 3)) as s3:
        q1, q2 = s3.residual(inp.t1, inp.t2)
        assert s3.slice_policy() == ((3, 3, 3), (None, None, None))
    assert all(x in (1, 2, 3) for x in sl) and min(sl) < 3
    assert all(e is not None and 0.0 <= e <= 1e-5 for e in err)
    # the probe measures at other amplitudes: allow a margin over the tolerance
    assert rel_err(r2, q2) < 1e-4 and rel_err(r1, q1) < 1e-4
    assert rel_err(r2, r2_ref) < 1e-4
    with _solver(inp, precision="mixed", slices=(0, 0, 0), slice_tolerance=1e-14) as s:
        assert s.slice_policy()[0] == (3, 3, 3)
    # measured at the amplitudes of the evaluation itself: each class within the
    # tolerance of 3 slices, so the residual within the sum of the three
    with _solver(inp, precision="mixed", slices=(0, 0, 0)) as s:
        sl2, err2 = s.calibrate_slices(inp.t1, inp.t2)
        c1, c2 = s.residual(inp.t1, inp.t2)
    assert all(e is not None and 0.0 <= e <= 1e-5 for e in err2)
    assert rel_err(c2, q2) <= 3e-5 and rel_err(c1, q1) <= 3e-5
    with _solver(inp, precision="mixed", slices=(3, 0, 1)) as s:
        sl, err = s.slice_policy()
        assert sl[0] == 3 and sl[2] == 1 and err[0] is None and err[2] is None and err[1] is not None


def test_mixed_solve_with_automatic_slices():
    inp = synth.make_inputs(8, 40, 40, seed=31, b_scale=0.02)
    ref = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, target_precision=1e-10, max_iter=60)
    with _solver(inp, precision="mixed", slices=(0, 0, 0), target_precision=1e-10, max_iter=60) as s:
        e, t1, t2, rep = s.solve()
    assert rep.converged and rep.fp64_iters >= 2
    assert abs(e - ref.e_corr) < 1e-6 and np.max(np.abs(t2 - ref.t2)) < 1e-6


def test_autotuned_tiles_give_the_same_residual():
    """The tuner only picks tile widths and K splits among candidates: the
    residual agrees with the untuned plan to rounding (K splits sum in FP64)."""
    inp = synth.make_inputs(10, 60, 30, seed=61, t1_scale=1e-2)
    with _solver(inp, precision="mixed", autotune=True) as s:
        a1, a2 = s.residual(inp.t1, inp.t2)
        prof = s.profile_residual()
    with _solver(inp, precision="mixed", autotune=False) as s:
        b1, b2 = s.residual(inp.t1, inp.t2)
    assert rel_err(a2, b2) < 1e-9 and rel_err(a1, b1) < 1e-9
    tc = [p for p in prof if p["pairs"] > 0]
    assert tc and all(p["bn"] in (32, 64, 128, 192, 256) and p["ksplit"] >= 1 for p in tc)


def test_residual_rejects_amplitudes_without_pair_symmetry():
    from mpqc_gb300._lib import GbccError
    inp = synth.make_inputs(4, 10, 12, seed=71, t1_scale=1e-2)
    bad = inp.t2.copy()
    bad[1, 2, 0, 3] += 1e-6
    with _solver(inp) as s:
        s.residual(inp.t1, inp.t2)
        with pytest.raises(GbccError) as e:
            s.residual(inp.t1, bad)
        assert e.value.status == 1 and "pair-symmetric" in str(e.value)
        r1, r2 = s.residual(inp.t1, inp.t2)   # the handle stays usable
    assert np.all(np.isfinite(r2))


def test_restart_from_checkpoint_converges_at_once(tmp_path):
    """gbcc_save_amplitudes / gbcc_load_amplitudes: a solve seeded with converged
    amplitudes stops after its first convergence test with the same energy."""
    inp = synth.make_inputs(5, 19, 30, seed=22)
    kw = dict(target_precision=1e-10, max_iter=40)
    with _solver(inp, **kw) as s:
        e0, t1, t2, rep0 = s.solve()
        path = tmp_path / "amps.bin"
        s.save_amplitudes(path)
    with _solver(inp, **kw) as s:
        assert abs(s.load_amplitudes(path) - e0) == 0.0
        e1, u1, u2, rep1 = s.solve()
    assert rep1.converged and rep1.iters <= 2 < rep0.iters
    assert abs(e1 - e0) < 1e-10 and np.max(np.abs(u2 - t2)) < 1e-9
    with _solver(inp, **kw) as s:
        with pytest.raises(L.GbccError) as ex:
            s.save_amplitudes(tmp_path / "none.bin")   # no solve yet
        assert ex.value.status == L.GBCC_ERR_STATE
        bad = t2.copy()
        bad[0, 1, 0, 0] += 1e-3                         # not pair-symmetric
        with pytest.raises(L.GbccError) as ex:
            s.set_amplitudes(t1, bad)
        assert ex.value.status == L.GBCC_ERR_INVALID_ARG
    with pytest.raises(L.GbccError) as ex:
        with Solver(4, 19) as s2:
            s2.set_inputs(inp.eps_o[:4], inp.eps_v, **{k: np.ascontiguousarray(v) for k, v in dict(
                Fia=inp.Fia[:4], Fij=inp.Fij[:4, :4], Fab=inp.Fab, Gijab=inp.Gijab[:4, :4], Gijkl=inp.Gijkl[:4, :4, :4, :4],
                Giajb=inp.Giajb[:4, :, :4], Gijka=inp.Gijka[:4, :4, :4], Giabc=inp.Giabc[:4], Gabcd=inp.Gabcd).items()})
            s2.load_amplitudes(path)                    # checkpoint of o = 5
    assert ex.value.status == L.GBCC_ERR_INVALID_ARG


@pytest.mark.parametrize("reset", [True, False])
def test_mixed_solve_refinement_with_and_without_diis_restart(reset):
    """The switch to FP64 refinement restarts the DIIS subspace (default) or keeps
    the split-precision vectors; both reach the oracle's energy within 1e-6 Eh."""
    inp = synth.make_inputs(6, 30, 40, seed=23)
    ref = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, target_precision=1e-9, max_iter=60)
    with _solver(inp, precision="mixed", slices=(2, 2, 2), target_precision=1e-9, max_iter=60,
                 refine_iters=2, refine_reset_diis=reset) as s:
        e, t1, t2, rep = s.solve()
    assert rep.converged and rep.fp64_iters >= 2
    assert abs(e - ref.e_corr) < 1e-6
    print(f"refine_reset_diis={reset}: {rep.mixed_iters} mixed + {rep.fp64_iters} FP64 iterations")
