"""GPU checks of gbcc_energy_noalloc, the allocation-free entry point.

It exists for callers that cannot allocate GPU memory when they test
convergence: a host framework that owns one fixed device pool and forbids
later allocation, or a caller that cannot accept the device-wide
synchronisation a cudaMalloc may cause.  They pass their own device arrays
and the library writes partial sums into a fixed __device__ array instead of
allocated scratch.  Its energy and residual error must match the oracle and
the handle-based gbcc_energy on the same amplitudes and residuals, on two
calls in a row (the second call reuses the scratch the first one left
behind), on a caller's own stream, and at v = 512, where the scratch is full.
This file is collected last so that a run stopping at its first failure has
already run every other test.
"""
import numpy as np
import pytest

from conftest import ints_dict

pytestmark = pytest.mark.gpu


def _oracle_energy(inp, r1, r2):
    """E = 2<f_ai + r1, t1> + <g_abij + r2, 2 tau - tau(b,a,i,j)> and
    sqrt(|r1|^2 + |r2|^2) / (n1 + n2) (ccsd.h:377-379, cc/solvers.h:60-63)."""
    from oracle import ccsd_ref as R
    tau = R.make_tau(inp.t1, inp.t2)
    g = inp.Gijab.transpose(2, 3, 0, 1)
    e = 2.0 * np.sum((inp.Fia.T + r1) * inp.t1) + np.sum((g + r2) * (2.0 * tau - tau.transpose(1, 0, 2, 3)))
    err = np.sqrt(np.sum(r1 * r1) + np.sum(r2 * r2)) / (r1.size + r2.size)
    return float(e), float(err), tau


def _noalloc(lib, torch, inp, r1, r2, tau, stream=None, calls=2):
    o, v = inp.o, inp.v

    def dev(x):
        return torch.from_numpy(np.ascontiguousarray(x)).cuda()

    f_ai, g_abij = dev(inp.Fia.T), dev(inp.Gijab.transpose(2, 3, 0, 1))
    t1, tau_d, r1_d, r2_d = dev(inp.t1), dev(tau), dev(r1), dev(r2)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    results = []
    for _ in range(calls):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        handle = None if stream is None else stream.cuda_stream
        st = lib.gbcc_energy_noalloc(o, v, f_ai.data_ptr(), g_abij.data_ptr(), t1.data_ptr(), tau_d.data_ptr(),
                                     r1_d.data_ptr(), r2_d.data_ptr(), out.data_ptr(), handle)
        assert st == 0, lib.gbcc_last_error(None)
        torch.cuda.synchronize()
        results.append(tuple(out.cpu().tolist()))
    return results


def _inputs(o, v, seed):
    """The arrays the energy reads: Fia, Gijab, pair-symmetric t1/t2, and
    residuals (random; the energy functional does not need the rest)."""
    from types import SimpleNamespace
    rng = np.random.default_rng(seed)
    Fia = rng.normal(0.0, 1e-2, (o, v))
    Gijab = rng.normal(0.0, 5e-2, (o, o, v, v))
    Gijab = 0.5 * (Gijab + Gijab.transpose(1, 0, 3, 2))
    t2 = rng.normal(0.0, 1e-2, (v, v, o, o))
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    t1 = rng.normal(0.0, 1e-2, (v, o))
    r1 = rng.normal(0.0, 1e-3, (v, o))
    r2 = rng.normal(0.0, 1e-3, (v, v, o, o))
    return SimpleNamespace(o=o, v=v, Fia=Fia, Gijab=Gijab, t1=t1, t2=t2), r1, r2


def _close(e, err, e_ref, err_ref):
    # the tolerance of the gbcc_energy check against the oracle
    assert abs(e - e_ref) < 1e-13 * max(1.0, abs(e_ref)), (e, e_ref)
    assert abs(err - err_ref) < 1e-15 + 1e-12 * err_ref, (err, err_ref)


def test_energy_noalloc_matches_oracle_and_gbcc_energy():
    torch = pytest.importorskip("torch")
    from mpqc_gb300 import Solver, _lib, build, synth
    build.build()
    lib = _lib.load()
    inp = synth.make_inputs(5, 23, 20, seed=77, t1_scale=1e-2)
    rng = np.random.default_rng(78)
    r1 = rng.normal(0.0, 1e-3, (23, 5))
    r2 = rng.normal(0.0, 1e-3, (23, 23, 5, 5))
    e_or, err_or, tau = _oracle_energy(inp, r1, r2)
    with Solver(inp.o, inp.v) as s:
        s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
        e_ref, err_ref = s.energy(inp.t1, inp.t2, r1, r2)
    _close(e_ref, err_ref, e_or, err_or)
    for e, err in _noalloc(lib, torch, inp, r1, r2, tau):
        _close(e, err, e_ref, err_ref)
        _close(e, err, e_or, err_or)


def test_energy_noalloc_on_a_caller_stream_at_the_scratch_limit():
    """v = 512 fills the 512 x 512 pair records exactly; the kernels run on
    the caller's own (non-default) stream."""
    torch = pytest.importorskip("torch")
    from mpqc_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    inp, r1, r2 = _inputs(1, 512, seed=91)
    e_or, err_or, tau = _oracle_energy(inp, r1, r2)
    stream = torch.cuda.Stream()
    for e, err in _noalloc(lib, torch, inp, r1, r2, tau, stream=stream):
        _close(e, err, e_or, err_or)


def test_energy_noalloc_rejects_sizes_and_host_pointers():
    """Sizes past the scratch limit and pointers that are not device memory
    are refused on the host, before any kernel is enqueued."""
    torch = pytest.importorskip("torch")
    from mpqc_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    o, v = 2, 3
    d = torch.zeros(v * v * o * o, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    assert lib.gbcc_energy_noalloc(o, 513, p, p, p, p, p, p, p, None) == _lib.GBCC_ERR_INVALID_ARG
    assert b"512" in lib.gbcc_last_error(None)
    host = np.zeros(2)
    st = lib.gbcc_energy_noalloc(o, v, p, p, p, p, p, p, host.ctypes.data, None)
    assert st == _lib.GBCC_ERR_INVALID_ARG
    assert b"not device memory" in lib.gbcc_last_error(None)
    assert host.tolist() == [0.0, 0.0]
