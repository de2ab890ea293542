"""CPU checks of the FP64 oracle: independent cross-check, structural
invariants of the reference equations, and the committed golden vectors."""
import numpy as np
import pytest

from conftest import load_golden, oracle_ints, rel_err
from mpqc_gb300 import synth
from oracle import ccsd_ref as R
from oracle import spinorb_ccsd as S


def _case(o, v, naux, seed, bs=0.05, t1s=1e-3):
    return synth.make_inputs(o, v, naux, seed=seed, b_scale=bs, t1_scale=t1s)


@pytest.mark.parametrize("o,v,naux,seed,bs", [(2, 4, 8, 1, 0.05), (3, 5, 10, 2, 0.08)])
def test_closed_shell_matches_spin_orbital_ccsd(o, v, naux, seed, bs):
    inp = synth.make_inputs(o, v, naux, seed=seed, b_scale=bs)
    B = synth.make_df_factor(np.random.default_rng(seed), naux, o + v, bs)
    Gfull = np.einsum("Qpr,Qqs->pqrs", B, B)
    res = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, target_precision=1e-12, max_iter=100)
    assert res.converged
    assert abs(res.e_corr - S.solve(inp.eps_o, inp.eps_v, Gfull)) < 1e-10
    # converged amplitudes make both residuals vanish
    r1, r2 = R.residual(res.t1, res.t2, oracle_ints(inp))
    assert np.max(np.abs(r1)) < 1e-8 and np.max(np.abs(r2)) < 1e-8


def test_r2_pair_symmetry():
    inp = _case(3, 6, 10, 5)
    r1, r2 = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    assert np.allclose(r2, r2.transpose(1, 0, 3, 2), atol=1e-15, rtol=0)


def test_zero_amplitudes_give_driver_terms():
    inp = _case(3, 5, 9, 6)
    o, v = inp.o, inp.v
    r1, r2 = R.residual(np.zeros((v, o)), np.zeros((v, v, o, o)), oracle_ints(inp))
    assert np.array_equal(r1, inp.Fia.T)
    assert np.allclose(r2, inp.Gijab.transpose(2, 3, 0, 1), atol=1e-15, rtol=0)


def test_first_jacobi_step_is_mp1():
    """From t = 0 the first update is t2 = g_abij / D (cf. mbpt/denom.h d_abij)."""
    inp = _case(3, 5, 9, 7)
    g = inp.Gijab.transpose(2, 3, 0, 1)
    t2 = R.jacobi_update_t2_abij(g, inp.eps_o, inp.eps_v)
    d = (inp.eps_o[None, None, :, None] + inp.eps_o[None, None, None, :]
         - inp.eps_v[:, None, None, None] - inp.eps_v[None, :, None, None])
    assert np.allclose(t2, g / d, rtol=1e-15, atol=0)
    res = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, max_iter=1)
    assert np.allclose(res.t2, g / d, rtol=1e-14, atol=0)


def test_reference_fvv_sign_matters_only_off_canonical():
    """The reference's 4-argument F_VV adds +f_ov(k,c) t1(a,k); with f_ov = 0
    (canonical orbitals) the energy equals spin-orbital CCSD, with f_ov != 0 it
    deviates.  The oracle and the CUDA path follow the reference as written."""
    o, v, naux, seed, bs = 2, 4, 8, 1, 0.05
    inp = synth.make_inputs(o, v, naux, seed=seed, b_scale=bs)
    rng = np.random.default_rng(7)
    n = o + v
    F = np.diag(np.concatenate([inp.eps_o, inp.eps_v]))
    X = rng.normal(0, 0.01, (n, n))
    F = F + X + X.T
    ints = oracle_ints(inp)
    ints.Fia, ints.Fij, ints.Fab = F[:o, o:].copy(), F[:o, :o].copy(), F[o:, o:].copy()
    e_ref = R.solve_ccsd(ints, np.diag(F)[:o].copy(), np.diag(F)[o:].copy(),
                         target_precision=1e-12, max_iter=200).e_corr
    orig = R.F_VV
    try:
        R.F_VV = lambda Fvv, fov, gb, t1: Fvv - R._es("kc,ak->ac", fov, t1) + R._es("kadc,dk->ac", gb, t1)
        e_fixed = R.solve_ccsd(ints, np.diag(F)[:o].copy(), np.diag(F)[o:].copy(),
                               target_precision=1e-12, max_iter=200).e_corr
    finally:
        R.F_VV = orig
    assert abs(e_ref - e_fixed) > 1e-7


def test_gepp_matches_lapack():
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 9):
        A = rng.normal(size=(n, n)) + n * np.eye(n)
        b = rng.normal(size=n)
        x, det = R.gepp_solve(A, b)
        assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-12, atol=1e-12)
        assert np.isclose(det, abs(np.linalg.det(A)), rtol=1e-10)
    assert R.gepp_solve(np.zeros((3, 3)), np.ones(3)) == (None, 0.0)


def test_diis_solves_linear_fixed_point():
    """Pulay DIIS on x = M x + c converges much faster than the plain iteration."""
    rng = np.random.default_rng(4)
    n = 30
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    M = Q @ np.diag(np.linspace(-0.9, 0.9, n)) @ Q.T
    c = rng.normal(size=n)
    exact = np.linalg.solve(np.eye(n) - M, c)
    d = R.PulayDIIS(ndiis=8)
    x = np.zeros(n)
    plain = np.zeros(n)
    for _ in range(40):
        xn = M @ x + c
        x = d.extrapolate([xn], [xn - x])[0]
        plain = M @ plain + c
    assert np.max(np.abs(x - exact)) < 1e-3 * np.max(np.abs(plain - exact))


def test_diis_group_and_start_parameters():
    d = R.PulayDIIS(start=3, ndiis=4)
    out = d.extrapolate([np.ones(2)], [np.ones(2)])
    assert d.last_coeffs is None and np.array_equal(out[0], np.ones(2))
    d2 = R.PulayDIIS(start=1, ndiis=2)
    for k in range(5):
        d2.extrapolate([np.full(2, float(k))], [np.full(2, 1.0 / (k + 1))])
    assert len(d2.xs) == 2 and d2.B.shape == (2, 2)


@pytest.mark.parametrize("name", ["residual_o3_v7", "residual_o5_v19"])
def test_golden_residuals(name):
    inp, g = load_golden(name)
    r1, r2 = R.residual(g["t1"], g["t2"], oracle_ints(inp))
    assert rel_err(r1, g["r1"]) < 1e-12
    assert rel_err(r2, g["r2"]) < 1e-12


def test_golden_solve():
    inp, g = load_golden("solve_o3_v8")
    res = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, target_precision=1e-11, max_iter=60)
    assert res.converged and res.iters == int(g["iters"])
    assert abs(res.e_corr - float(g["e_corr"])) < 1e-12
    assert rel_err(res.t2, g["t2"]) < 1e-9


def test_flop_count_matches_contraction_list():
    # the synthetic o=32, v=320 residual: 3.53e13 FLOP (61 % ladder)
    f = R.flop_count(32, 320)
    assert abs(f - 3.53e13) / 3.53e13 < 0.01
    assert abs(2 * 32**2 * 320**4 / f - 0.61) < 0.01
    assert synth.flop_count(5, 19) == R.flop_count(5, 19)


def test_sampled_residual_time_tracks_the_full_residual():
    """The CPU baseline's bounded sample (every contraction of the oracle's
    residual, operands in the oracle's memory orders, on a slab of its first
    output index, scaled back) estimates the time of the full residual.  It
    leaves out the array additions between contractions, so it reads low:
    measured 0.54-0.61 of the full time at o = 12..16, v = 48..96."""
    import time
    from mpqc_gb300 import synth
    from oracle import ccsd_sample as S
    tr = S.trace()
    assert len(tr) > 40 and any(spec == "cdij,abcd->abij" for spec, _, _ in tr)
    o, v = 12, 48
    inp = synth.make_inputs(o, v, 40, seed=1, t1_scale=1e-3)
    ints = R.Integrals(inp.Fia, inp.Fij, inp.Fab, inp.Gijab, inp.Gijkl, inp.Giajb, inp.Gijka, inp.Giabc,
                       inp.Gabcd)
    R.residual(inp.t1, inp.t2, ints)
    full = min(_timed(lambda: R.residual(inp.t1, inp.t2, ints), time) for _ in range(3))
    est = min(S.sampled_seconds(o, v, 0.5, tr)[0] for _ in range(3))
    assert 0.35 * full < est < 1.5 * full, (full, est)


def _timed(fn, time):
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0


def test_direct_branches_equal_the_standard_residual():
    """The integral-direct branches of the oracle (U of ccsd.h:581-603 used at
    ccsd_r1_r2.h:116-118, 282-286) are an exact rearrangement of the standard
    residual when the MO blocks come from the same AO integrals."""
    from oracle import molecule as M
    from mpqc_gb300 import molecules
    sym, xyz = molecules.water()
    mol = M.Molecule(sym, molecules.to_bohr(xyz))
    S, H, G = M.ao_integrals_c(mol, "6-31G")
    scf = M.rhf(S, H, G, 5, mol.nuclear_repulsion())
    blocks, eo, ev = M.mo_blocks(scf, G, 1)
    o, v = len(eo), len(ev)
    rng = np.random.default_rng(2)
    t2 = rng.normal(0.0, 1e-2, (v, v, o, o))
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    t1 = rng.normal(0.0, 1e-2, (v, o))
    r1, r2 = R.residual(t1, t2, R.Integrals(**blocks))
    ints = R.Integrals(**blocks, Ci=scf.C[:, 1:5], Ca=scf.C[:, 5:])
    d1, d2 = R.residual(t1, t2, ints, G_ao=G)
    assert rel_err(d1, r1) < 1e-13 and rel_err(d2, r2) < 1e-13
