"""Bounded-sample timing of the oracle's residual at a full configuration.

TEST AND BENCHMARK INFRASTRUCTURE ONLY (the CPU-baseline and reference legs
of bench.py, and tests/).  It measures how long the FP64 oracle
(oracle/ccsd_ref.py, the CPU restatement of the reference's R1 + R2) would
take for one residual at sizes too large to run within a benchmark step
(o = 32, v = 320: the (ab|cd) block alone is 84 GB and the residual about a
minute of multi-core BLAS time), without building the full problem:

* ``trace()`` runs ``ccsd_ref.residual`` once at a tiny size (o = 3, v = 7)
  and records every einsum contraction it performs -- index specification
  and, per operand, which dimensions are occupied and which virtual, and the
  operand's memory order (the oracle passes transposed views of its
  integrals, which einsum copies);
* ``sampled_seconds(o, v, frac)`` replays each recorded contraction with
  operands of the full shapes and the same memory orders, except that the
  first index of its output is cut to a slab of ``frac`` of its range (a
  contraction's cost is linear in each output index), times it, and scales
  the time back by the slab fraction.  The sum estimates one full residual.

The operand values are a constant (timing only).  Array additions and
scalings between the contractions (a few O(o^2 v^2) passes, about a quarter
of the oracle's time at o = 16, v = 96) are not included.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import ccsd_ref as R

_O_SMALL, _V_SMALL = 3, 7


def trace():
    """[(spec, [operand dims as 'o'/'v' strings])] of one oracle residual."""
    from mpqc_gb300 import synth
    rec = []
    orig = R._es

    def recording(spec, *ops):
        kinds = ["".join("o" if d == _O_SMALL else "v" for d in op.shape) for op in ops]
        # axes from the slowest-varying in memory to the fastest
        orders = [tuple(int(a) for a in np.argsort([-st for st in op.strides], kind="stable")) for op in ops]
        rec.append((spec, kinds, orders))
        return orig(spec, *ops)

    inp = synth.make_inputs(_O_SMALL, _V_SMALL, 5, seed=3, t1_scale=1e-2)
    ints = R.Integrals(inp.Fia, inp.Fij, inp.Fab, inp.Gijab, inp.Gijkl, inp.Giajb, inp.Gijka, inp.Giabc,
                       inp.Gabcd)
    R._es = recording
    try:
        R.residual(inp.t1, inp.t2, ints)
    finally:
        R._es = orig
    return rec


def sampled_seconds(o, v, frac=1.0 / 32, contractions=None):
    """Estimated seconds of one oracle residual at (o, v) and the per-
    contraction details [(spec, sampled seconds, scale)]."""
    contractions = contractions if contractions is not None else trace()
    dims = {"o": o, "v": v}
    total, details = 0.0, []
    for spec, kinds, orders in contractions:
        ins, out = spec.split("->")
        labels = ins.split(",")
        first = out[0] if out else None
        ops, scale = [], 1.0
        for lab, kind, order in zip(labels, kinds, orders):
            shape = [dims[k] for k in kind]
            if first is not None and first in lab:
                ax = lab.index(first)
                w = max(1, math.ceil(shape[ax] * frac))
                scale = shape[ax] / w
                shape[ax] = w
            # contiguous in the recorded memory order, viewed in the logical order
            base = np.full([shape[a] for a in order], 1e-3)
            ops.append(base.transpose(np.argsort(order)))
        t0 = time.perf_counter()
        np.einsum(spec, *ops, optimize=True)
        dt = time.perf_counter() - t0
        total += dt * scale
        details.append((spec, dt, scale))
        del ops
    return total, details
