"""The process-wide autotune table on the GPU: a handle whose contraction
shapes are in the table (from an earlier handle, or loaded from a file)
times no candidate tile, and computes with exactly the recorded tiles."""
import ctypes as C

import numpy as np
import pytest

from conftest import ints_dict
from mpqc_gb300 import Solver, _lib, autotune_clear, autotune_load, autotune_save, synth

pytestmark = pytest.mark.gpu


def _tc_launches(lib, s):
    n = C.c_int64()
    assert lib.gbcc_testing_tc_launches_total(s.h, C.byref(n)) == 0
    return n.value


def test_autotune_table_reuse(tmp_path):
    lib = _lib.load()
    inp = synth.make_inputs(16, 72, 40, seed=7, t1_scale=1e-2)
    autotune_clear()
    try:
        with Solver(inp.o, inp.v, precision="mixed", slices=(2, 2, 2), autotune=True) as s:
            s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
            timed = _tc_launches(lib, s)
            r1a, r2a = s.residual(inp.t1, inp.t2)
        assert timed > 0
        path = tmp_path / "tune.txt"
        autotune_save(path)
        assert len(path.read_text().splitlines()) > 1
        autotune_clear()
        autotune_load(path)
        with Solver(inp.o, inp.v, precision="mixed", slices=(2, 2, 2), autotune=True) as s:
            s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))
            assert _tc_launches(lib, s) == 0
            r1b, r2b = s.residual(inp.t1, inp.t2)
        assert np.array_equal(r1a, r1b) and np.array_equal(r2a, r2b)
    finally:
        autotune_clear()


def test_nvtx_ranges_leave_results_unchanged(tmp_path):
    """GBCC_NVTX=1 wraps every operation of a residual in an NVTX range named
    by the operation; a residual with the ranges on (direct launches, a fresh
    process, tiles from the planner's heuristic so that both processes use the
    same ones) equals one without them bit for bit."""
    import os
    import subprocess
    import sys
    from conftest import ROOT
    script = tmp_path / "nvtx_residual.py"
    script.write_text(
        "import sys, numpy as np\n"
        f"sys.path.insert(0, {str(ROOT)!r}); sys.path.insert(0, {str(ROOT / 'tests')!r})\n"
        "from conftest import ints_dict\n"
        "from mpqc_gb300 import Solver, synth\n"
        "inp = synth.make_inputs(6, 30, 20, seed=4, t1_scale=1e-2)\n"
        "with Solver(inp.o, inp.v, precision='mixed', slices=(2, 2, 2), use_graphs=0, autotune=False) as s:\n"
        "    s.set_inputs(inp.eps_o, inp.eps_v, **ints_dict(inp))\n"
        "    r1, r2 = s.residual(inp.t1, inp.t2)\n"
        "np.save(sys.argv[1], np.concatenate([r1.ravel(), r2.ravel()]))\n")
    out = {}
    for flag in ("0", "1"):
        env = dict(os.environ, GBCC_NVTX=flag)
        f = tmp_path / f"r_{flag}.npy"
        r = subprocess.run([sys.executable, str(script), str(f)], env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        out[flag] = np.load(f)
    assert np.array_equal(out["0"], out["1"])
