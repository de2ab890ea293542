"""Generate the committed golden fixtures from the FP64 oracle.

The reference's own tests pin only total energies of molecular inputs whose
AO integrals and basis data are not available here, and hold no
amplitude-level vectors.  These fixtures therefore freeze the oracle (itself
cross-checked against an independent spin-orbital CCSD) on seeded synthetic
inputs, so regressions of either the oracle or the CUDA path show up as a
mismatch against a file.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from mpqc_gb300 import synth  # noqa: E402
from oracle import ccsd_ref as R  # noqa: E402

CASES = {
    # name: (o, v, naux, seed, b_scale, t2_scale, t1_scale)
    "residual_o3_v7": (3, 7, 12, 11, 0.05, 1e-2, 1e-3),
    "residual_o5_v19": (5, 19, 40, 12, 0.05, 1e-2, 1e-3),
    "solve_o3_v8": (3, 8, 14, 13, 0.05, 0.0, 0.0),
}


def ints_of(inp):
    return R.Integrals(inp.Fia, inp.Fij, inp.Fab, inp.Gijab, inp.Gijkl, inp.Giajb, inp.Gijka,
                       inp.Giabc, inp.Gabcd)


def main():
    for name, (o, v, naux, seed, bs, t2s, t1s) in CASES.items():
        rng = np.random.default_rng(seed)
        B = synth.make_df_factor(rng, naux, o + v, bs)
        eps_o = np.sort(rng.uniform(-1.5, -0.3, size=o))
        eps_v = np.sort(rng.uniform(0.1, 3.0, size=v))
        t2 = rng.normal(0.0, t2s or 1e-2, size=(v, v, o, o))
        t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
        t1 = rng.normal(0.0, t1s, size=(v, o)) if t1s > 0 else np.zeros((v, o))
        inp = synth.inputs_from_factor(B, eps_o, eps_v, t1, t2)
        ints = ints_of(inp)
        # inputs are stored as the DF factor; tests rebuild the integral blocks
        data = dict(o=o, v=v, naux=naux, seed=seed, B=B, eps_o=eps_o, eps_v=eps_v)
        if name.startswith("residual"):
            r1, r2 = R.residual(inp.t1, inp.t2, ints)
            data.update(t1=inp.t1, t2=inp.t2, r1=r1, r2=r2)
        else:
            res = R.solve_ccsd(ints, inp.eps_o, inp.eps_v, target_precision=1e-11, max_iter=60)
            assert res.converged
            data.update(e_corr=res.e_corr, t1=res.t1, t2=res.t2, iters=res.iters,
                        energies=np.array([h[3] for h in res.history]))
        np.savez_compressed(HERE / f"{name}.npz", **data)
        print(name, "written")


if __name__ == "__main__":
    main()
