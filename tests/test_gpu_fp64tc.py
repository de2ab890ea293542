"""FP64-grade contractions on the BF16 tensor cores (GBCC_PREC_FP64_TC).

Each operand row is held in six 8-bit fixed-point slices under the row's
largest exponent; the slice products of one weight class are integers of a
common scale, so their FP32 sums in TMEM are exact, and the classes are
accumulated in float-float and FP64.  Checked here:
  * the packed slices bit for bit against a numpy restatement of the split;
  * exactness: on inputs whose product is exact in FP64, the tensor-core
    result equals numpy's bit for bit;
  * accuracy on random data against the 2^-46 K rowmax(A) rowmax(B) bound;
  * residuals and whole solves against the FP64 oracle and the FP64 path."""
import ctypes as C

import numpy as np
import pytest

from conftest import ints_dict, load_golden, load_molecule, oracle_ints, rel_err
from mpqc_gb300 import Solver, synth
from oracle import ccsd_ref as R

pytestmark = pytest.mark.gpu

NSL = 6


def _bf16_bits(I, base):
    """BF16 bits of I 2^k, |I| <= 256, biased exponent of 2^k = base (flush below range)."""
    out = np.zeros(I.shape, dtype=np.uint16)
    nz = I != 0
    a = np.abs(I[nz]).astype(np.int64)
    L = np.floor(np.log2(a)).astype(np.int64)
    be = base[nz] + L
    mant = np.where(L <= 7, a << np.maximum(7 - L, 0), a >> np.maximum(L - 7, 0)) & 0x7F
    sign = np.where(I[nz] < 0, 0x8000, 0)
    val = np.where(be <= 0, sign, sign | (np.clip(be, 0, 255) << 7) | mant)
    val = np.where(be >= 255, sign | 0x7F80, val)
    out[nz] = val.astype(np.uint16)
    return out


def fixed_split_np(x, n=NSL):
    """Restatement of the packing kernels' fixed-point split, row by row."""
    u = x.view(np.uint64)
    e = ((u >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    e_row = np.where(e == 0x7FF, 0, e).max(axis=1)
    m = ((u & np.uint64(0xFFFFFFFFFFFFF)) | np.uint64(1 << 52)).astype(np.int64)
    sh = 54 + (e_row[:, None] - e) - 8 * n
    X = np.zeros(x.shape, dtype=np.int64)
    ok = (e != 0) & (e != 0x7FF) & (e_row[:, None] != 0) & (sh <= 62)
    shs = np.where(ok, sh, 1)
    X = np.where(ok, (m + (np.int64(1) << (shs - 1))) >> shs, 0)
    X = np.where(x < 0, -X, X)
    digits = [None] * n
    for p in range(n - 1, 0, -1):
        r = ((X + 128) & 255) - 128
        digits[p] = r
        X = (X - r) >> 8
    digits[0] = X
    out = np.stack([_bf16_bits(digits[p], np.broadcast_to(e_row[:, None] - 902 - 8 * p, x.shape))
                    for p in range(n)])
    return out, e_row


def _bf16_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def tlib(gbcc_lib):
    return gbcc_lib


def _fixed_split_gpu(tlib, x, n=NSL):
    rows, cols = x.shape
    out = np.zeros((n, rows, cols), dtype=np.uint16)
    re = np.zeros(rows, dtype=np.uint32)
    x = np.ascontiguousarray(x)
    assert tlib.gbcc_testing_fixed_split(x.ctypes.data, rows, cols, n, out.ctypes.data, re.ctypes.data) == 0
    return out, re


@pytest.mark.parametrize("rows,cols", [(1, 1), (3, 70), (130, 200), (257, 64)])
def test_fixed_split_bits_match_restatement(tlib, rows, cols):
    rng = np.random.default_rng(rows * 1000 + cols)
    x = rng.normal(size=(rows, cols)) * np.exp(rng.uniform(-30, 30, size=(rows, 1)))
    x *= np.exp(rng.uniform(-8, 0, size=(rows, cols)))  # small elements next to the row maximum
    x[rng.random(size=x.shape) < 0.1] = 0.0
    if rows > 2:
        x[1] = 0.0                                      # an all-zero row
        x[2, 0] = 1e-310                                # a subnormal
    got, re = _fixed_split_gpu(tlib, x)
    ref, re_ref = fixed_split_np(x)
    assert np.array_equal(re, re_ref.astype(np.uint32))
    assert np.array_equal(got, ref)
    # the slices sum to x within half a unit of the last digit of the row
    recon = _bf16_to_f64(got).sum(axis=0)
    E = re_ref.astype(np.int64) - 1022
    bound = np.ldexp(1.0, E - 8 * NSL)[:, None]
    assert np.all(np.abs(recon - x) <= bound)


def _gemm_tc(tlib, A, B, bn=0, ksplit=1, repeat=1, cta2=0):
    M, K = A.shape
    N = B.shape[0]
    Cm = np.zeros((M, N))
    ms = C.c_float()
    st = tlib.gbcc_testing_gemm_fp64tc(M, N, K, np.ascontiguousarray(A).ctypes.data,
                                       np.ascontiguousarray(B).ctypes.data, Cm.ctypes.data, bn, ksplit, cta2, repeat,
                                       C.byref(ms))
    assert st == 0
    return Cm, ms.value


@pytest.mark.parametrize("M,N,K,bn,ksplit,cta2", [(128, 128, 1000, 0, 1, 0), (200, 70, 1500, 64, 1, 0),
                                                  (64, 300, 4096, 128, 4, 0), (5, 9, 64, 32, 1, 0),
                                                  (300, 200, 2000, 128, 1, 1), (520, 64, 777, 64, 1, 1)])
def test_fp64tc_exact_where_the_product_is_exact(tlib, M, N, K, bn, ksplit, cta2):
    """Integers of at most 21 (A) and 16 (B) bits, scaled by per-row powers
    of two: every product and partial sum is exact in FP64, and the fixed
    point holds them without rounding, so the result must equal numpy's bit
    for bit -- which holds only if every TMEM chunk sum is exact."""
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-(1 << 20), 1 << 20, size=(M, K)).astype(np.float64)
    B = rng.integers(-(1 << 15), 1 << 15, size=(N, K)).astype(np.float64)
    A *= np.ldexp(1.0, rng.integers(-20, 20, size=(M, 1)))
    B *= np.ldexp(1.0, rng.integers(-20, 20, size=(N, 1)))
    Cg, _ = _gemm_tc(tlib, A, B, bn, ksplit, cta2=cta2)
    assert np.array_equal(Cg, A @ B.T)


@pytest.mark.parametrize("M,N,K,ksplit", [(256, 192, 2048, 1), (300, 100, 12880, 6), (1024, 512, 777, 1)])
def test_fp64tc_accuracy_bound(tlib, M, N, K, ksplit):
    rng = np.random.default_rng(K)
    A = rng.normal(size=(M, K)) * np.exp(rng.uniform(-5, 5, size=(M, 1)))
    B = rng.normal(size=(N, K)) * np.exp(rng.uniform(-5, 5, size=(N, 1)))
    Cg, _ = _gemm_tc(tlib, A, B, 0, ksplit)
    ref = A @ B.T
    bound = 2.0 ** -46 * K * np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=1)[None, :]
    err = np.abs(Cg - ref)
    print(f"M={M} N={N} K={K}: max err/bound {np.max(err / bound):.2e}, rel {rel_err(Cg, ref):.2e}")
    assert np.all(err <= bound)
    # 47 bits below each row's leading power of two: ~2^-47 of rowmax x rowmax
    # (measured 0.8e-13 to 1.3e-13 of max|C| on these inputs)
    assert rel_err(Cg, ref) < 5e-13


def _solver(inp, precision, **kw):
    s = Solver(inp.o, inp.v, precision=precision, slices=(3, 3, 3), **kw)
    s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
    return s


@pytest.mark.parametrize("name", ["residual_o3_v7", "residual_o5_v19"])
def test_fp64tc_residual_golden(name):
    inp, g = load_golden(name)
    with _solver(inp, "fp64_tc") as s:
        r1, r2 = s.residual(g["t1"], g["t2"])
    assert rel_err(r1, g["r1"]) < 1e-12
    assert rel_err(r2, g["r2"]) < 1e-12


@pytest.mark.parametrize("o,v,naux", [(8, 40, 30), (16, 72, 40), (12, 130, 60)])
def test_fp64tc_residual_random(o, v, naux):
    inp = synth.make_inputs(o, v, naux, seed=o * 10 + v, t1_scale=1e-2)
    r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    with _solver(inp, "fp64_tc") as s:
        r1, r2 = s.residual(inp.t1, inp.t2)
        f1, f2 = s.residual(inp.t1, inp.t2, precision="fp64")
    e1, e2 = rel_err(r1, r1_ref), rel_err(r2, r2_ref)
    print(f"o={o} v={v} fp64_tc: r2 {e2:.2e}, r1 {e1:.2e}")
    assert e1 < 1e-12 and e2 < 1e-12
    assert rel_err(f2, r2_ref) < 1e-12


def test_mixed_handle_takes_fp64tc_residuals_only_when_planned():
    inp = synth.make_inputs(4, 12, 10, seed=5, t1_scale=1e-2)
    from mpqc_gb300._lib import GBCC_ERR_STATE, GbccError
    with _solver(inp, "mixed") as s:
        with pytest.raises(GbccError) as ex:
            s.residual(inp.t1, inp.t2, precision="fp64_tc")
        assert ex.value.status == GBCC_ERR_STATE
    with _solver(inp, "mixed", refine_precision="fp64_tc") as s:
        r1, r2 = s.residual(inp.t1, inp.t2, precision="fp64_tc")
    r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    assert rel_err(r2, r2_ref) < 1e-11 and rel_err(r1, r1_ref) < 1e-11


@pytest.mark.parametrize("name,frozen,key", [("h2o_631g", False, "ref_e_ccsd"), ("h2o_ccpvdz", True, "ref_e_ccsd_fc")])
def test_fp64tc_solve_reproduces_recorded_energy(name, frozen, key):
    """The reference's recorded water energies (its own CPU runs)."""
    from conftest import freeze_first_occupied
    blocks, eo, ev, g = load_molecule(name)
    if frozen:
        blocks, eo = freeze_first_occupied(blocks, eo)
    with Solver(len(eo), len(ev), precision="fp64_tc", target_precision=1e-11, max_iter=60) as s:
        s.set_inputs(eo, ev, **blocks)
        e, _, _, rep = s.solve(want_amplitudes=False)
    assert rep.converged and rep.mixed_iters == 0
    assert abs(e - float(g[key])) <= float(g["precision"])


def test_mixed_solve_with_fp64tc_refinement_matches_fp64():
    inp = synth.make_inputs(8, 40, 40, seed=31, b_scale=0.02)
    ref = R.solve_ccsd(oracle_ints(inp), inp.eps_o, inp.eps_v, target_precision=1e-10, max_iter=60)
    out = {}
    for rp in ("fp64", "fp64_tc"):
        with _solver(inp, "mixed", target_precision=1e-10, max_iter=60, refine_iters=2, refine_precision=rp) as s:
            e, t1, t2, rep = s.solve()
        assert rep.converged and rep.mixed_iters > 0 and rep.fp64_iters >= 2
        out[rp] = (e, t2, rep)
    assert abs(out["fp64_tc"][0] - ref.e_corr) < 1e-9
    assert abs(out["fp64_tc"][0] - out["fp64"][0]) < 1e-10
    assert out["fp64_tc"][2].iters == out["fp64"][2].iters
