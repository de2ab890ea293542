"""Time one GEMM shape on the library's kernels (profiling aid).

    python -m mpqc_gb300.gemm_probe M N K [--slices 2] [--bn 0] [--ksplit 1]
                                      [--cta2 0] [--sps 1] [--group 1] [--cmode 0] [--repeat 5]
                                      [--chunk 0] [--check]

Runs C = A B^T on seeded normal FP64 inputs through gbcc_testing_gemm_ex3
(split-BF16 tensor-core kernel for slices >= 1, plain FP64 for 0) and prints
one JSON line: the kernel time per launch and the executed slice-product
TFLOP/s.  The launches are what an ncu capture of this command sees
(``-k regex:gemm_tc_kernel``).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("M", type=int)
    ap.add_argument("N", type=int)
    ap.add_argument("K", type=int)
    ap.add_argument("--slices", type=int, default=2)
    ap.add_argument("--bn", type=int, default=0)
    ap.add_argument("--ksplit", type=int, default=1)
    ap.add_argument("--cta2", type=int, default=0)
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--sps", type=int, default=1, help="slices per pipeline stage (2: both slices)")
    ap.add_argument("--group", type=int, default=1, help="M tiles per band of the tile order (1: whole rows)")
    ap.add_argument("--cmode", type=int, default=0,
                    help="output form: bit 0 accumulate into C (beta = 1), bit 1 C unit-stride along M")
    ap.add_argument("--repeat", type=int, default=5)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--check", action="store_true",
                    help="also report max |C - A B^T| / max |A B^T| against numpy FP64")
    a = ap.parse_args(argv)
    from mpqc_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(a.seed)
    A = rng.normal(size=(a.M, a.K))
    B = rng.normal(size=(a.N, a.K))
    Cm = np.empty((a.M, a.N))
    ms = C.c_float()
    st = lib.gbcc_testing_gemm_ex3(a.M, a.N, a.K, A.ctypes.data, B.ctypes.data, Cm.ctypes.data, a.slices,
                                   a.ksplit, a.bn, a.cta2, a.chunk, 0, a.sps, a.group, a.cmode, a.repeat,
                                   C.byref(ms))
    pairs = a.slices * (a.slices + 1) // 2 if a.slices > 0 else 1
    flops = 2.0 * a.M * a.N * a.K
    out = {"M": a.M, "N": a.N, "K": a.K, "slices": a.slices, "bn": a.bn, "ksplit": a.ksplit, "cta2": a.cta2,
           "sps": a.sps, "group": a.group, "cmode": a.cmode, "chunk": a.chunk,
           "status": st, "ms": ms.value,
           "executed_tflops": pairs * flops / (ms.value * 1e-3) / 1e12 if st == 0 and ms.value > 0 else None}
    if a.check and st == 0:
        ref = A @ B.T
        out["max_rel_err"] = float(np.max(np.abs(Cm - ref)) / np.max(np.abs(ref)))
    print(json.dumps(out), flush=True)
    return 0 if st == 0 else 1


if __name__ == "__main__":
    raise SystemExit(main())
