"""GPU checks of the two GEMM kernels in isolation (FP64 DFMA kernel and the
split-BF16 tcgen05 kernel) against a NumPy FP64 product, through the
library's test hook."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (128, 64, 64), (200, 100, 70), (300, 33, 500), (129, 257, 1000), (64, 256, 128),
          (1000, 32, 40), (96, 1024, 64)]

# max |C - C_ref| / max |C_ref| allowed per slice count (0 = FP64 kernel)
TOL = {0: 1e-13, 1: 3e-2, 2: 2e-4, 3: 5e-6}


@pytest.fixture(scope="module")
def tlib(gbcc_lib):
    lib = gbcc_lib
    lib.gbcc_testing_gemm.restype = C.c_int
    lib.gbcc_testing_gemm.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_int, C.c_int, C.POINTER(C.c_float)]
    lib.gbcc_testing_fp64_peak.restype = C.c_int
    lib.gbcc_testing_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    return lib


def run(tlib, A, B, slices):
    M, K = A.shape
    N = B.shape[0]
    out = np.empty((M, N))
    ms = C.c_float()
    st = tlib.gbcc_testing_gemm(M, N, K, A.ctypes.data, B.ctypes.data, out.ctypes.data, slices, 1, C.byref(ms))
    assert st == 0, st
    return out


@pytest.mark.parametrize("slices", [0, 1, 2, 3])
@pytest.mark.parametrize("M,N,K", SHAPES)
def test_gemm_matches_fp64(tlib, M, N, K, slices):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.normal(size=(M, K)) * np.exp(rng.uniform(-3, 3, size=(M, K)))
    B = rng.normal(size=(N, K))
    ref = A @ B.T
    out = run(tlib, A, B, slices)
    scale = np.max(np.abs(ref))
    # split products accumulate in FP32: allow the sqrt(K) growth of its rounding
    tol = TOL[slices] + (8 * 2.0**-24 * np.sqrt(K) if slices else 0.0)
    assert np.max(np.abs(out - ref)) <= tol * scale


def test_gemm_repeat_is_deterministic(tlib):
    rng = np.random.default_rng(1)
    A = rng.normal(size=(257, 300))
    B = rng.normal(size=(130, 300))
    assert np.array_equal(run(tlib, A, B, 3), run(tlib, A, B, 3))


def test_fp64_probe_runs(tlib):
    g = C.c_double()
    assert tlib.gbcc_testing_fp64_peak(C.byref(g)) == 0
    assert g.value > 10.0
    d = C.c_double()
    assert tlib.gbcc_testing_dmma_peak(C.byref(d)) == 0
    assert d.value > 10.0
    print(f"FP64 DFMA {g.value:.0f} GFLOP/s, DMMA {d.value:.0f} GFLOP/s")


@pytest.mark.parametrize("slices", [0, 3])
@pytest.mark.parametrize("M,N,K,ksplit", [(32, 32, 20000, 37), (320, 32, 9000, 9), (5, 7, 4096, 64),
                                          (200, 130, 3000, 3)])
def test_gemm_split_k(tlib, M, N, K, ksplit, slices):
    rng = np.random.default_rng(K + ksplit)
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K))
    ref = A @ B.T
    out = np.empty((M, N))
    ms = C.c_float()
    st = tlib.gbcc_testing_gemm_ex(M, N, K, A.ctypes.data, B.ctypes.data, out.ctypes.data, slices, ksplit,
                                   0, 0, 0, 0, 1, C.byref(ms))
    assert st == 0
    tol = TOL[slices] + (8 * 2.0**-24 * np.sqrt(K) if slices else 0.0)
    assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref))
    out2 = np.empty((M, N))
    tlib.gbcc_testing_gemm_ex(M, N, K, A.ctypes.data, B.ctypes.data, out2.ctypes.data, slices, ksplit,
                              0, 0, 0, 0, 1, C.byref(ms))
    assert np.array_equal(out, out2)


# kernel variants: (bn, cta2, chunk, fold); bn 192 and 256 sum chunks in FP32 registers
VARIANTS = [(256, 0, 4, 0), (256, 0, 8, 0), (192, 0, 4, 0), (128, 1, 4, 16), (64, 1, 4, 16), (128, 0, 1, 1),
            (64, 0, 16, 64)]


@pytest.mark.parametrize("bn,cta2,chunk,fold", VARIANTS)
@pytest.mark.parametrize("M,N,K,ksplit", [(256, 256, 64, 1), (300, 520, 1000, 1), (700, 300, 2000, 3),
                                          (128, 256, 6000, 5), (260, 528, 1500, 1)])
def test_gemm_kernel_variants(tlib, M, N, K, ksplit, bn, cta2, chunk, fold):
    rng = np.random.default_rng(M + N + K + bn)
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K))
    ref = A @ B.T
    out = np.empty((M, N))
    ms = C.c_float()
    st = tlib.gbcc_testing_gemm_ex(M, N, K, A.ctypes.data, B.ctypes.data, out.ctypes.data, 3, ksplit, bn, cta2,
                                   chunk, fold, 1, C.byref(ms))
    assert st == 0
    # FP32 accumulation of the chunks (bn 256) grows like sqrt(number of chunks)
    tol = TOL[3] + 8 * 2.0**-24 * np.sqrt(K)
    assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref))


@pytest.mark.parametrize("bn", [64, 128, 192])
@pytest.mark.parametrize("M,N,K,ksplit", [(256, 256, 64, 1), (300, 520, 1000, 1), (260, 528, 1500, 1),
                                          (700, 300, 2000, 3)])
def test_gemm_both_slices_per_stage(tlib, M, N, K, ksplit, bn):
    """Two slices staged together (one stage per k-block feeding all three pair
    products) against FP64: the same sums as one pair per stage."""
    rng = np.random.default_rng(M + N + K + bn + 7)
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K))
    ref = A @ B.T
    out = np.empty((M, N))
    out1 = np.empty((M, N))
    ms = C.c_float()
    tlib.gbcc_testing_gemm_ex2.restype = C.c_int
    tlib.gbcc_testing_gemm_ex2.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p] + \
        [C.c_int] * 8 + [C.POINTER(C.c_float)]
    st = tlib.gbcc_testing_gemm_ex2(M, N, K, A.ctypes.data, B.ctypes.data, out.ctypes.data, 2, ksplit, bn, 0, 0, 0,
                                    2, 1, C.byref(ms))
    st1 = tlib.gbcc_testing_gemm_ex2(M, N, K, A.ctypes.data, B.ctypes.data, out1.ctypes.data, 2, ksplit, bn, 0, 0,
                                     0, 1, 1, C.byref(ms))
    assert st == 0 and st1 == 0
    tol = TOL[2] + 8 * 2.0**-24 * np.sqrt(K)
    assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref))
    assert np.max(np.abs(out - out1)) <= 2 * tol * np.max(np.abs(ref))


@pytest.mark.parametrize("bn,sps", [(192, 2), (256, 1), (128, 1)])
@pytest.mark.parametrize("M,N,K,group,ksplit", [(2000, 1700, 640, 8, 1), (1500, 1900, 512, 8, 1),
                                                (1500, 1900, 512, 3, 1), (900, 1300, 2048, 8, 2)])
def test_gemm_banded_tile_order(tlib, M, N, K, group, ksplit, bn, sps):
    """Output tiles run in bands of `group` M tiles (the last band short where
    the M tiles do not divide): the same tiles in another order, so the
    result equals the row-order one bit for bit."""
    rng = np.random.default_rng(M + N + K + group + bn)
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K))
    ms = C.c_float()
    tlib.gbcc_testing_gemm_ex3.restype = C.c_int
    tlib.gbcc_testing_gemm_ex3.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p] + \
        [C.c_int] * 10 + [C.POINTER(C.c_float)]
    outs = []
    for g in (1, group):
        out = np.empty((M, N))
        st = tlib.gbcc_testing_gemm_ex3(M, N, K, A.ctypes.data, B.ctypes.data, out.ctypes.data, 2, ksplit, bn, 0, 0,
                                        0, sps, g, 0, 1, C.byref(ms))
        assert st == 0
        outs.append(out)
    assert np.array_equal(outs[0], outs[1])
    ref = A @ B.T
    tol = TOL[2] + 8 * 2.0**-24 * np.sqrt(K)
    assert np.max(np.abs(outs[1] - ref)) <= tol * np.max(np.abs(ref))


@pytest.mark.parametrize("slices,bn,sps", [(2, 192, 2), (2, 256, 1), (2, 64, 1), (0, 0, 1)])
@pytest.mark.parametrize("cmode", [1, 2, 3])
@pytest.mark.parametrize("ksplit", [1, 3])
def test_gemm_output_forms(tlib, slices, bn, sps, cmode, ksplit):
    """Accumulating epilogue (beta = 1) and column-major C (the m-major
    epilogue) give the product of the row-major, beta = 0 form."""
    M, N, K = 700, 900, 384
    rng = np.random.default_rng(cmode * 10 + slices + bn + ksplit)
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K))
    ms = C.c_float()
    tlib.gbcc_testing_gemm_ex3.restype = C.c_int
    tlib.gbcc_testing_gemm_ex3.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p] + \
        [C.c_int] * 10 + [C.POINTER(C.c_float)]
    outs = []
    for mode in (0, cmode):
        out = np.empty((M, N))
        st = tlib.gbcc_testing_gemm_ex3(M, N, K, A.ctypes.data, B.ctypes.data, out.ctypes.data, slices, ksplit, bn,
                                        0, 0, 0, sps, 1, mode, 2, C.byref(ms))
        assert st == 0
        outs.append(out)
    # beta = 1 on zeros and a column-major store change no bits of the product
    assert np.array_equal(outs[0], outs[1])
    ref = A @ B.T
    tol = (TOL[slices] + 8 * 2.0**-24 * np.sqrt(K)) if slices else TOL[0]
    assert np.max(np.abs(outs[1] - ref)) <= tol * np.max(np.abs(ref))


def test_bounded_wait_returns_a_timeout_and_the_context_stays_usable(tlib):
    """Failure detection without a GPU fault: the producer leaves one stage of
    every CTA unloaded and the barriers' wait limit is 1 ms, so the MMA
    thread's bounded wait runs out; the kernel records GBCC_ERR_TIMEOUT,
    drains its copies, waits for its MMAs, frees its tensor memory and
    returns.  The same product then runs normally, and so does a residual
    through a handle (tensor memory was given back, the context is intact)."""
    from mpqc_gb300 import Solver, synth
    from mpqc_gb300._lib import GBCC_ERR_TIMEOUT
    from oracle import ccsd_ref as R
    from conftest import ints_dict, oracle_ints, rel_err
    lib = tlib
    rng = np.random.default_rng(5)
    M, N, K = 256, 256, 1024                   # 4 tiles; 16 k-blocks x 6 slice pairs each
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K))
    out = np.zeros((M, N))
    first, second = C.c_int(-1), C.c_int(-1)
    st = lib.gbcc_testing_gemm_timeout(M, N, K, A.ctypes.data, B.ctypes.data, out.ctypes.data, 1_000_000, 3,
                                       C.byref(first), C.byref(second))
    assert st == 0
    assert first.value == GBCC_ERR_TIMEOUT and second.value == 0
    ref = A @ B.T
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 5e-6
    inp = synth.make_inputs(4, 12, 10, seed=11, t1_scale=1e-2)
    with Solver(inp.o, inp.v, precision="mixed", slices=(3, 3, 3)) as s:
        s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
        r1, r2 = s.residual(inp.t1, inp.t2)
    r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    assert rel_err(r2, r2_ref) < 2e-6 and rel_err(r1, r1_ref) < 2e-6
