"""GPU check of gbcc_energy_noalloc, the allocation-free entry point.

It exists for callers that cannot allocate GPU memory when they test
convergence (a host framework that owns a fixed device pool, or a stream
being captured into a CUDA graph): they pass their own device arrays and the
library writes partial sums into a fixed __device__ array instead of
allocated scratch.  Its energy and residual error must match the
handle-based gbcc_energy on the same amplitudes and residuals, on two calls
in a row (the second call reuses the scratch the first one left behind).
This file is collected last so that a run stopping at its first failure has
already run every other test.
"""
import numpy as np
import pytest

from conftest import ints_dict

pytestmark = pytest.mark.gpu


def test_energy_noalloc_matches_gbcc_energy():
    torch = pytest.importorskip("torch")
    from mpqc_gb300 import Solver, _lib, build, synth
    build.build()
    lib = _lib.load()
    o, v = 5, 23
    inp = synth.make_inputs(o, v, 20, seed=77, t1_scale=1e-2)
    rng = np.random.default_rng(5)
    r1 = rng.normal(0.0, 1e-3, (v, o))
    r2 = rng.normal(0.0, 1e-3, (v, v, o, o))
    with Solver(o, v) as s:
        s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
        e_ref, err_ref = s.energy(inp.t1, inp.t2, r1, r2)

    def dev(x):
        return torch.from_numpy(np.ascontiguousarray(x)).cuda()

    tau = inp.t2 + np.einsum("ai,bj->abij", inp.t1, inp.t1)
    f_ai, g_abij = dev(inp.Fia.T), dev(inp.Gijab.transpose(2, 3, 0, 1))
    t1, tau_d, r1_d, r2_d = dev(inp.t1), dev(tau), dev(r1), dev(r2)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        st = lib.gbcc_energy_noalloc(o, v, f_ai.data_ptr(), g_abij.data_ptr(), t1.data_ptr(), tau_d.data_ptr(),
                                     r1_d.data_ptr(), r2_d.data_ptr(), out.data_ptr(), None)
        assert st == 0, lib.gbcc_last_error(None)
        torch.cuda.synchronize()
        e, err = out.cpu().tolist()
        # same tolerance as the gbcc_energy check against the oracle
        assert abs(e - e_ref) < 1e-13 * max(1.0, abs(e_ref))
        assert abs(err - err_ref) < 1e-15 + 1e-12 * err_ref
