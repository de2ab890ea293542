"""Failure paths made on the host (no GPU fault): an allocation that fails as
if the device were full, inside the tensors' creation and inside the
set-up that follows it; and the DIIS coefficient solve on singular B."""
import ctypes as C

import numpy as np
import pytest

from conftest import ints_dict, oracle_ints, rel_err
from mpqc_gb300 import Solver, _lib, synth
from mpqc_gb300._lib import GBCC_ERR_OOM, GBCC_ERR_STATE, GbccError
from oracle import ccsd_ref as R

pytestmark = pytest.mark.gpu


def _diis(lib, B, damping=0.0):
    n = B.shape[0]
    B = np.ascontiguousarray(B, dtype=np.float64)
    coef = np.zeros(n)
    nskip = C.c_int32()
    assert lib.gbcc_testing_diis_coefficients(n, B.ctypes.data, damping, coef.ctypes.data, C.byref(nskip)) == 0
    return coef, nskip.value


def test_diis_coefficients_regular_and_singular():
    lib = _lib.load()
    rng = np.random.default_rng(3)
    E = rng.normal(size=(4, 50))
    B = E @ E.T
    coef, nskip = _diis(lib, B)
    A = np.zeros((5, 5))
    A[0, 1:] = A[1:, 0] = -1.0
    A[1:, 1:] = B
    ref = np.linalg.solve(A, np.r_[-1.0, np.zeros(4)])[1:]
    assert nskip == 0 and abs(coef.sum() - 1.0) < 1e-12 and np.allclose(coef, ref, rtol=1e-10, atol=1e-12)
    # the two oldest error vectors equal: B is singular, the oldest is dropped
    E2 = E.copy()
    E2[1] = E2[0]
    coef, nskip = _diis(lib, E2 @ E2.T)
    assert nskip >= 1 and np.all(np.isfinite(coef)) and abs(coef.sum() - 1.0) < 1e-12 and coef[0] == 0.0
    # every stored vector the same: only the newest is kept
    ones = np.ones((3, 3))
    coef, nskip = _diis(lib, ones)
    assert nskip == 2 and np.array_equal(coef, [0.0, 0.0, 1.0])


def _fail_after(lib, n):
    count = C.c_int64()
    assert lib.gbcc_testing_fail_alloc(n, C.byref(count)) == 0
    return count.value


def test_allocation_failure_leaves_usable_state():
    lib = _lib.load()
    inp = synth.make_inputs(4, 12, 10, seed=11, t1_scale=1e-2)
    r1_ref, r2_ref = R.residual(inp.t1, inp.t2, oracle_ints(inp))
    try:
        # a failure while the handle's tensors are created: the handle refuses
        # further calls (its tensors are incomplete) and is destroyed cleanly
        with Solver(inp.o, inp.v, precision="fp64") as s:
            _fail_after(lib, 2)
            with pytest.raises(GbccError) as ex:
                s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
            assert ex.value.status == GBCC_ERR_OOM and "injected" in str(ex.value)
            _fail_after(lib, -1)
            with pytest.raises(GbccError) as ex:
                s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
            assert ex.value.status == GBCC_ERR_STATE
        # how many allocations a complete set-up makes
        with Solver(inp.o, inp.v, precision="fp64") as s:
            c0 = _fail_after(lib, -1)
            s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
            n = _fail_after(lib, -1) - c0
        assert n > 30
        # a failure in the set-up after the tensors exist: the same handle takes
        # the inputs again and evaluates the residual
        with Solver(inp.o, inp.v, precision="fp64") as s:
            _fail_after(lib, n - 1)
            with pytest.raises(GbccError) as ex:
                s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
            assert ex.value.status == GBCC_ERR_OOM
            _fail_after(lib, -1)
            s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
            r1, r2 = s.residual(inp.t1, inp.t2)
        assert rel_err(r1, r1_ref) < 1e-12 and rel_err(r2, r2_ref) < 1e-12
    finally:
        _fail_after(lib, -1)
