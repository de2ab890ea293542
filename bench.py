"""Benchmark: CCSD residual throughput on one GB300 (one JSON line on stdout).

Workload: the synthetic CCSD doubles residual -- one R1 + R2 evaluation, no
molecule -- with o = 32 occupied and v = 320 virtual orbitals and a density-
fitted integral set of naux = 1200 auxiliary functions.  The integrals are
built on the device from a seeded DF factor B[Q,p,q] ~ N(0, 0.05) (symmetrised)
as <pq|rs> = sum_Q B[Q,p,r] B[Q,q,s] (the v^4 block (ab|cd) alone is 84 GB in
FP64); t2 ~ N(0, 1e-2) symmetrised, t1 ~ N(0, 1e-3); eps_occ ~ U(-1.5,-0.3),
eps_virt ~ U(0.1,3.0).  Inputs (about 150 GB touched per residual) exceed the
129 MB L2 many times over, so no L2 flush is needed between steps.

Reported (one JSON line):
  value      algorithmic TFLOP/s of the mixed-precision residual, F(o,v) / (s/iter),
             F = 2o^2v^4 + 12o^3v^3 + 4o^4v^2 + 14o^2v^3 + 18o^3v^2, inputs resident in HBM
  e2e        the same through the C ABI with host (pinned) t1/t2 in and r1/r2 out
  fp64       the plain-FP64 (DFMA) residual on the same inputs (s/iter, TFLOP/s)
  fp64_tc    the FP64-grade residual on the tensor cores (fixed-point slices) on
             the same inputs, with its speed-up and max|dr2| against plain FP64
  roofline   the particle-particle ladder GEMM (dominant kernel) against the BF16 tensor peak
  cpu_baseline  the FP64 oracle on the host cores at the same o, v: each of the
             residual's contractions timed on a slab of its first output index
             and scaled back (oracle/ccsd_sample.py)

--impl reference times the FP64 CPU oracle (the restatement of the reference's
CPU path; the reference itself cannot be built here) the same way, on the
same workload and config as this arm.
--config h2o10 runs (H2O)10 / cc-pVDZ from the geometry (mixed, FP64-grade
tensor-core and FP64 solves, and the (T) correction of the mixed solve).
--config batch64 solves 64 water clusters (H2O)1..6 together (clusters/s).
Multi-GPU (torchrun): every rank runs an independent replica ("replicas only",
weak scaling); value = sum of all ranks' FLOPs / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "CCSD s/iter and residual TFLOP/s, mixed vs plain-FP64 on 1 GB300 at |ΔE|≤1e-6 Eh"


def flop_count(o, v):
    return 2 * o**2 * v**4 + 12 * o**3 * v**3 + 4 * o**4 * v**2 + 14 * o**2 * v**3 + 18 * o**3 * v**2


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value, ws, device="cpu"):
    """The largest value over the ranks of the job; every rank receives it."""
    if ws <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(flops_per_step, ms_step, ws):
    """TFLOP/s of ws replicas that each evaluate flops_per_step per step, the step
    time being the slowest rank's."""
    return ws * flops_per_step / (ms_step * 1e-3) / 1e12


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# CPU baseline / reference arm: the FP64 oracle on a bounded sample

def cpu_threads():
    try:
        from threadpoolctl import threadpool_info
        n = [i.get("num_threads") for i in threadpool_info() if i.get("user_api") == "blas"]
        if n:
            return int(max(n))
    except Exception:
        pass
    return os.cpu_count() or 1


def bench_config(args, ws):
    """The workload both arms report (identical dicts)."""
    return {"workload": "synthetic CCSD doubles residual, one R1+R2 evaluation",
            "o": args.o, "v": args.v, "naux": args.naux, "parallelism": f"replicas{ws}",
            "flops_per_step": flop_count(args.o, args.v), "l2": "inputs larger than L2 (no flush)"}


def cpu_sampled_rate(o, v, frac, steps, warmup):
    """TFLOP/s of the FP64 oracle's residual at (o, v), each step a bounded
    sample: every contraction of the residual at its full shapes with the
    first output index cut to a slab of `frac` (oracle/ccsd_sample.py),
    scaled back by the slab fraction."""
    from oracle import ccsd_sample as S
    tr = S.trace()
    for _ in range(warmup):
        S.sampled_seconds(o, v, frac, tr)
    est = [S.sampled_seconds(o, v, frac, tr)[0] for _ in range(max(1, steps))]
    sec = float(np.median(est))
    return flop_count(o, v) / sec / 1e12, sec


def cpu_sample_text(o, v, frac):
    return (f"FP64 oracle residual (numpy/OpenBLAS restatement of the reference's R1+R2) at o={o} v={v}: "
            f"each of its 55 contractions timed at full shapes with the first output index cut to "
            f"1/{round(1 / frac)} of its range, scaled back; array additions between contractions not timed")


def reference_arm(args):
    ws, rank, _ = dist_env()
    if ws > 1 and rank != 0:
        return 0
    rate, sec = cpu_sampled_rate(args.o, args.v, args.cpu_frac, max(1, args.steps), max(0, args.warmup))
    line = {
        "metric": METRIC, "value": rate, "unit": "TFLOP/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": bench_config(args, ws),
        "cpu_baseline": {"value": rate, "unit": "TFLOP/s", "cores": cpu_threads(), "kind": "port",
                         "sample": cpu_sample_text(args.o, args.v, args.cpu_frac)},
        "e2e": {"value": rate, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# device-side input generation

class _DevArray:
    """Zero-copy torch view of a device buffer owned by the library."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(int(s) for s in shape), "typestr": "<f8",
                                         "data": (int(ptr), False), "version": 3, "strides": None}


def build_inputs(torch, solver, o, v, naux, seed, dev, b_scale=0.05):
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    n = o + v
    B = torch.randn((naux, n, n), generator=g, device=dev, dtype=torch.float64) * b_scale
    B = (B + B.transpose(1, 2)) * (0.5 ** 0.5)
    eps_o = torch.sort(torch.rand(o, generator=g, device=dev, dtype=torch.float64) * 1.2 - 1.5).values
    eps_v = torch.sort(torch.rand(v, generator=g, device=dev, dtype=torch.float64) * 2.9 + 0.1).values
    t2 = torch.randn((v, v, o, o), generator=g, device=dev, dtype=torch.float64) * 1e-2
    t2 = 0.5 * (t2 + t2.permute(1, 0, 3, 2))
    t1 = torch.randn((v, o), generator=g, device=dev, dtype=torch.float64) * 1e-3
    ptr = solver.device_inputs()
    view = lambda name, shape: torch.as_tensor(_DevArray(ptr[name], shape), device=dev)  # noqa: E731
    view("eps_o", (o,)).copy_(eps_o)
    view("eps_v", (v,)).copy_(eps_v)
    view("Fia", (o, v)).zero_()
    view("Fij", (o, o)).copy_(torch.diag(eps_o))
    view("Fab", (v, v)).copy_(torch.diag(eps_v))
    Boo, Bov, Bvv = B[:, :o, :o], B[:, :o, o:], B[:, o:, o:]

    def blk(x, y):  # <pq|rs> = sum_Q x[Q,p,r] y[Q,q,s], in FP64
        return torch.einsum("Qpr,Qqs->pqrs", x, y)

    view("Gijab", (o, o, v, v)).copy_(blk(Bov, Bov))
    view("Gijkl", (o, o, o, o)).copy_(blk(Boo, Boo))
    view("Giajb", (o, v, o, v)).copy_(blk(Boo, Bvv))
    view("Gijka", (o, o, o, v)).copy_(blk(Boo, Bov))
    Giabc = view("Giabc", (o, v, v, v))
    for i in range(o):
        Giabc[i].copy_(torch.einsum("Qr,Qqs->qrs", Bov[:, i, :], Bvv))
    Gabcd = view("Gabcd", (v, v, v, v))
    Y = Bvv.reshape(naux, v * v)                      # (Q, b d)
    step = 8
    for a0 in range(0, v, step):
        a1 = min(v, a0 + step)
        X = Bvv[:, a0:a1, :].permute(1, 2, 0).reshape((a1 - a0) * v, naux)   # (a c, Q)
        P = (X @ Y).reshape(a1 - a0, v, v, v)                                # (a, c, b, d)
        Gabcd[a0:a1].copy_(P.permute(0, 2, 1, 3))
    del X, Y, P, B
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    solver.commit_inputs()
    return t1.contiguous(), t2.contiguous()


# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"gbcc_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        try:
            rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.strip()]
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if len(r) > 5 + k and "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


def ncu_traffic():
    """Per-launch DRAM bytes of the ladder GEMM from the committed ncu summary."""
    p = ROOT / "profiles" / "ladder_gemm_o32_v320.md"
    try:
        for line in p.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except Exception:
        pass
    return None


def ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from mpqc_gb300 import build as gb
    gb.build()
    from mpqc_gb300 import Solver, autotune_load, autotune_save
    if args.autotune_table and os.path.exists(args.autotune_table):
        autotune_load(args.autotune_table)
    o, v, naux = args.o, args.v, args.naux
    F = flop_count(o, v)
    log(f"[bench] rank {rank}: building inputs o={o} v={v} naux={naux} on {torch.cuda.get_device_name(dev)}")
    t_setup = time.perf_counter()
    s = Solver(o, v, precision="mixed", slices=(args.slices,) * 3, autotune=not args.no_autotune, device=local)
    t1, t2 = build_inputs(torch, s, o, v, naux, args.seed, dev,
                          b_scale=0.05 if args.b_scale is None else args.b_scale)
    log(f"[bench] inputs + split packing ready in {time.perf_counter() - t_setup:.1f} s")
    # slice counts per term class from the error measured at this workload's
    # amplitudes (fewest slices within 1e-5 of the 3-slice residual)
    slices_used, slice_err = s.calibrate_slices(t1, t2)
    log(f"[bench] slices (ladder, ring, other) = {slices_used}, rel. change vs 3 slices = {slice_err}")
    if args.autotune_table:
        autotune_save(args.autotune_table)
    r1 = torch.empty_like(t1)
    r2 = torch.empty_like(t2)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    if args.residual_only:
        # profiling driver: warmup + steps mixed residuals and nothing else;
        # reports which tensor-core GEMM launch of a residual is the ladder and
        # how many tensor-core launches (calibration, tuning) came before
        tc_before = s.tc_launches_total()
        for _ in range(args.warmup + args.steps):
            s.residual(t1, t2, r1, r2, precision="mixed")
        torch.cuda.synchronize()
        prof = s.profile_residual(precision="mixed")
        tc = [p for p in prof if p["pairs"] > 0]
        ordinal = next(i for i, p in enumerate(tc) if p["cls"] == 0)
        launches = s.last_launches()
        s.close()
        if rank == 0:
            print(json.dumps({"residual_only": True, "o": o, "v": v, "naux": naux,
                              "tc_launches_per_residual": len(tc), "ladder_tc_ordinal": ordinal,
                              "launches_per_residual": launches,
                              "tc_launches_before_first_residual": tc_before,
                              "ladder_ncu_skip": tc_before + ordinal,
                              "tc_sites_mnk_class": [[p["M"], p["N"], p["K"], p["cls"]] for p in tc]}),
                  flush=True)
        return 0

    # ---- mixed precision, device-resident inputs
    for _ in range(args.warmup):
        s.residual(t1, t2, r1, r2, precision="mixed")
    launches = s.last_launches()
    barrier()
    with ClockSampler(local) as clk:
        s.record(0)
        for _ in range(args.steps):
            s.residual(t1, t2, r1, r2, precision="mixed")
        s.record(1)
        ms = s.elapsed_ms(0, 1)
    barrier()
    ms_step = max_over_ranks(ms / args.steps, ws, dev)
    value = whole_job_rate(F, ms_step, ws)
    r2_mixed = r2.clone()

    # ---- end to end through the C ABI: pinned host buffers, copies inside the timed region
    h_t1 = torch.empty(t1.shape, dtype=torch.float64, pin_memory=True)
    h_t2 = torch.empty(t2.shape, dtype=torch.float64, pin_memory=True)
    h_r1 = torch.empty(t1.shape, dtype=torch.float64, pin_memory=True)
    h_r2 = torch.empty(t2.shape, dtype=torch.float64, pin_memory=True)
    h_t1.copy_(t1)
    h_t2.copy_(t2)
    a_t1, a_t2, a_r1, a_r2 = (x.numpy() for x in (h_t1, h_t2, h_r1, h_r2))
    s.residual(a_t1, a_t2, a_r1, a_r2, precision="mixed")
    barrier()
    e2e_steps = max(1, args.steps)
    s.record(2)
    for _ in range(e2e_steps):
        s.residual(a_t1, a_t2, a_r1, a_r2, precision="mixed")
    s.record(3)
    e2e_ms = max_over_ranks(s.elapsed_ms(2, 3) / e2e_steps, ws, dev)
    e2e_value = whole_job_rate(F, e2e_ms, ws)
    bytes_io = (t1.numel() + t2.numel()) * 8

    # ---- per-term profile and roofline of the dominant kernel (ladder GEMM)
    prof = s.profile_residual(precision="mixed")
    pk = peaks()
    ladder = [p for p in prof if p["cls"] == 0]
    roof = None
    if ladder and ladder[0]["gemm_ms"] > 0:
        lp = ladder[0]
        executed = lp["pairs"] * lp["flops"]
        peak = pk.get("bf16_tflops_sustained") or 1700.0
        ach = executed / (lp["gemm_ms"] * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                "traffic": ncu_traffic(),
                "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of this launch "
                                  "(profiles/ladder_gemm_o32_v320.md), not measured in this run",
                "kernel": "gemm_tc_kernel (particle-particle ladder, G+ tau+ pair products)",
                "executed_flops_per_launch": executed, "launch_ms": lp["gemm_ms"],
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"}
    terms = {}
    for p in prof:
        key = {0: "ladder", 1: "ring", 2: "other", -1: "elementwise"}[p["cls"]]
        terms[key] = terms.get(key, 0.0) + p["ms"]

    s.close()

    # ---- plain FP64 (DFMA) and FP64-grade tensor-core residuals on the same
    # inputs, from a second handle (its fixed-point slice packs and the mixed
    # ones together would not fit in HBM at v = 320)
    fp64 = fp64_tc = None
    if args.fp64_steps > 0 or not args.no_fp64_tc:
        s = Solver(o, v, precision="fp64" if args.no_fp64_tc else "fp64_tc", device=local)
        build_inputs(torch, s, o, v, naux, args.seed, dev, b_scale=0.05 if args.b_scale is None else args.b_scale)
        r2_fp64 = None
        if args.fp64_steps > 0:
            s.residual(t1, t2, r1, r2, precision="fp64")
            barrier()
            s.record(4)
            for _ in range(args.fp64_steps):
                s.residual(t1, t2, r1, r2, precision="fp64")
            s.record(5)
            f_ms = s.elapsed_ms(4, 5) / args.fp64_steps
            err = float((r2_mixed - r2).abs().max() / r2.abs().max())
            fp64 = {"s_per_iter": f_ms * 1e-3, "tflops": F / (f_ms * 1e-3) / 1e12, "steps": args.fp64_steps,
                    "warmup": 1, "mixed_speedup": f_ms / ms_step,
                    "mixed_vs_fp64_max_rel_err_r2": err}
            r2_fp64 = r2.clone()
        if not args.no_fp64_tc:
            s.residual(t1, t2, r1, r2, precision="fp64_tc")
            barrier()
            s.record(6)
            for _ in range(args.steps):
                s.residual(t1, t2, r1, r2, precision="fp64_tc")
            s.record(7)
            c_ms = s.elapsed_ms(6, 7) / args.steps
            fp64_tc = {"s_per_iter": c_ms * 1e-3, "tflops": F / (c_ms * 1e-3) / 1e12, "steps": args.steps,
                       "warmup": 1, "dtype": "fixed-point bf16x6 (8-bit digits under each row's exponent), exact "
                                             "FP32 class sums, float-float chunks, f64 I/O"}
            if r2_fp64 is not None:
                fp64_tc["speedup_vs_fp64"] = fp64["s_per_iter"] / fp64_tc["s_per_iter"]
                fp64_tc["max_rel_err_r2_vs_fp64"] = float((r2 - r2_fp64).abs().max() / r2_fp64.abs().max())
        s.close()

    if rank != 0:
        return 0
    cpu = None
    if not args.no_cpu:
        rate, sec = cpu_sampled_rate(o, v, args.cpu_frac, 1, 1)
        cpu = {"value": rate, "unit": "TFLOP/s", "cores": cpu_threads(), "kind": "port",
               "sample": cpu_sample_text(o, v, args.cpu_frac) + f" ({sec:.1f} s per residual estimated)"}
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "s_per_iter": ms_step * 1e-3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        # the arithmetic of the contractions: FP64 operands split into BF16
        # slices, FP32 tensor-core accumulation, FP64 in and out
        "dtype": f"split-bf16x{max(slices_used)} (f64 I/O)",
        "data": "synthetic",
        "config": bench_config(args, ws),
        "precision_policy": {"slices_ladder_ring_other": list(slices_used),
                             "slice_rel_change_vs_3": list(slice_err),
                             "accumulation": "FP32 TMEM chunks, float-float or FP32 register fold, FP64 epilogue"},
        "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": bytes_io,
                "d2h_bytes_per_step": bytes_io, "ms_per_step": e2e_ms},
        "fp64": fp64,
        "fp64_tc": fp64_tc,
        "roofline": roof,
        "term_ms": terms,
        "gpu_launches": launches * args.steps,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def solve_report(args):
    """Whole Jacobi+DIIS solves from t = 0 on one synthetic input: mixed precision
    (split-BF16 bulk contractions, then refinement iterations in --refine
    precision) and plain FP64, with s/iter of each and the mixed result's
    |dE_corr| and max|dT2| against the FP64 one."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    from mpqc_gb300 import build as gb
    gb.build()
    from mpqc_gb300 import Solver
    o, v, naux = args.o, args.v, args.naux
    # random DF factors give a pair correlation energy of about 0.45 v^2 naux b^4;
    # this scale puts it near 1.5e-3 Eh (real molecules: ~1e-3 Eh per pair)
    bs = (3.0e-3 / (v * v * naux)) ** 0.25 if args.b_scale is None else args.b_scale
    F = flop_count(o, v)
    runs, amps = {}, {}
    for prec in ("mixed",) if args.no_solve_fp64 else ("mixed", "fp64"):
        s = Solver(o, v, precision=prec, slices=(args.slices,) * 3, target_precision=args.solve_precision,
                   max_iter=args.max_iter, refine_iters=2, refine_precision=args.refine)
        build_inputs(torch, s, o, v, naux, args.seed, dev, b_scale=bs)
        sl_used, sl_err = s.slice_policy()
        t0 = time.perf_counter()
        e, t1, t2, rep = s.solve()
        wall = time.perf_counter() - t0
        s.close()
        sm, sf = rep.seconds_residual_mixed, rep.seconds_residual_fp64
        runs[prec] = {"e_corr": e, "converged": rep.converged, "iters": rep.iters,
                      "mixed_iters": rep.mixed_iters, "fp64_iters": rep.fp64_iters,
                      "seconds_total": wall,
                      "s_per_iter_mixed": sm or None, "s_per_iter_fp64": sf or None,
                      "tflops_mixed": F / sm / 1e12 if sm else None,
                      "tflops_fp64": F / sf / 1e12 if sf else None}
        if prec == "mixed":
            runs[prec]["slices"] = list(sl_used)
            runs[prec]["slice_rel_change_vs_3"] = list(sl_err)
        amps[prec] = (t1, t2)
        log(f"[solve] {prec}: E={e:.12f} iters={rep.iters} ({rep.mixed_iters} mixed) "
            f"converged={rep.converged} {wall:.1f} s")
    line = {"solve": True, "o": o, "v": v, "naux": naux, "b_scale": bs, "seed": args.seed,
            "flops_per_iter": F, "target_precision": args.solve_precision, "refine_precision": args.refine,
            "runs": runs,
            "data": "synthetic DF-factored integrals, B ~ N(0, b_scale), t = 0 start"}
    if "fp64" in runs:
        m, f = runs["mixed"], runs["fp64"]
        line["abs_dE_mixed_vs_fp64"] = abs(m["e_corr"] - f["e_corr"])
        line["max_abs_dT2_mixed_vs_fp64"] = float(np.max(np.abs(amps["mixed"][1] - amps["fp64"][1])))
        line["max_abs_dT1_mixed_vs_fp64"] = float(np.max(np.abs(amps["mixed"][0] - amps["fp64"][0])))
        if m["s_per_iter_mixed"] and f["s_per_iter_fp64"]:
            line["per_iteration_speedup"] = f["s_per_iter_fp64"] / m["s_per_iter_mixed"]
        line["solve_speedup"] = f["seconds_total"] / m["seconds_total"]
    print(json.dumps(line), flush=True)
    return 0


def molecule_report(args):
    """The (H2O)10 / cc-pVDZ target on the GPU, from the geometry: AO integrals,
    RHF and the AO -> MO transform on the device, then three solves on the
    same MO integrals: mixed precision (split-BF16 bulk contractions, FP64
    denominators, DIIS, energy, then two refinement iterations in
    --refine precision), FP64-grade on the tensor cores throughout (fp64_tc),
    and plain FP64 (DFMA).  Reports |dE_corr| of each against the FP64
    oracle's energy (tests/golden/h2o10_ccpvdz.json, computed on the CPU by
    tests/golden/make_h2o10.py), max|dT2| against the FP64 solve, s/iter and
    TFLOP/s of each path, and the ladder GEMM's fraction of the BF16 peak."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    from mpqc_gb300 import build as gb
    gb.build()
    from mpqc_gb300 import RHF, Solver, molecules
    nw = args.waters
    sym, xyz = molecules.water_cluster(nw, seed=0)
    fixture = ROOT / "tests" / "golden" / ("h2o10_ccpvdz.json" if nw == 10 else f"h2o{nw}_ccpvdz.json")
    ref = json.loads(fixture.read_text()) if fixture.exists() else None
    t0 = time.perf_counter()
    scf = RHF(sym, xyz, "cc-pVDZ", threshold=1e-11, max_iter=60)
    e_scf = scf.run()
    srep = scf.report
    nocc = scf.nocc()
    o, v = nocc, scf.nbf - nocc
    F = flop_count(o, v)
    log(f"[h2o{nw}] N={scf.nbf} o={o} v={v}: E_RHF {e_scf:.10f} ({srep.iters} it., ERI {srep.seconds_eri:.2f} s, "
        f"SCF {srep.seconds_scf:.2f} s, wall {time.perf_counter() - t0:.1f} s)")
    if args.scf_only:
        # profiling aid: the input producer alone (integrals, RHF)
        print(json.dumps({"molecule": f"(H2O){nw}", "basis": "cc-pVDZ", "nbf": srep.nbf, "e_rhf": e_scf,
                          "scf": {"iters": srep.iters, "eri_s": srep.seconds_eri, "scf_s": srep.seconds_scf,
                                  "one_body_s": srep.seconds_one_body}}), flush=True)
        scf.close()
        return 0
    runs, amps = {}, {}
    for prec in ("mixed", "fp64_tc") if args.no_solve_fp64 else ("mixed", "fp64_tc", "fp64"):
        s = Solver(o, v, precision=prec, target_precision=args.solve_precision, max_iter=args.max_iter,
                   refine_iters=2, refine_precision=args.refine)
        t1 = time.perf_counter()
        scf.ccsd_inputs(s)
        t_in = time.perf_counter() - t1
        t2_ = time.perf_counter()
        e, a1, a2, rep = s.solve()
        wall = time.perf_counter() - t2_
        # inputs_s: the MO transform on the device and the input commit (slice
        # calibration and autotuning in mixed precision)
        run = {"e_corr": e, "converged": rep.converged, "iters": rep.iters, "mixed_iters": rep.mixed_iters,
               "fp64_iters": rep.fp64_iters, "solve_s": wall, "inputs_s": t_in,
               "s_per_iter_mixed": rep.seconds_residual_mixed or None,
               "s_per_iter_fp64": rep.seconds_residual_fp64 or None}
        if prec == "mixed" or (prec == "fp64_tc" and args.triples_fp64_tc):
            # (T) of the converged amplitudes on this handle, in the solve's arithmetic
            t3 = time.perf_counter()
            e_t = s.triples("mixed" if prec == "mixed" else "fp64_tc")
            run["triples"] = {"e_t": e_t, "seconds": time.perf_counter() - t3,
                              "precision": "mixed" if prec == "mixed" else "fp64_tc"}
            log(f"[h2o{nw}] (T) {run['triples']['precision']}: {e_t:.12f} in {run['triples']['seconds']:.1f} s")
        if prec == "mixed":
            sl, se = s.slice_policy()
            run["slices"], run["slice_rel_change_vs_3"] = list(sl), list(se)
            prof = s.profile_residual(precision="mixed")
            lad = [p for p in prof if p["cls"] == 0 and p["gemm_ms"] > 0]
            if lad:
                lp = max(lad, key=lambda p: p["flops"])
                ach = lp["pairs"] * lp["flops"] / (lp["gemm_ms"] * 1e-3) / 1e12
                pk = peaks().get("bf16_tflops") or 1953.9
                run["ladder"] = {"M": lp["M"], "N": lp["N"], "K": lp["K"], "launch_ms": lp["gemm_ms"],
                                 "executed_tflops": ach, "frac_of_bf16_burst_peak": ach / pk}
            run["term_ms"] = {}
            for p in prof:
                key = {0: "ladder", 1: "ring", 2: "other", -1: "elementwise"}[p["cls"]]
                run["term_ms"][key] = run["term_ms"].get(key, 0.0) + p["ms"]
        s.close()
        runs[prec] = run
        amps[prec] = a2
        log(f"[h2o{nw}] {prec}: E_corr {e:.12f}, {rep.iters} it. ({rep.mixed_iters} mixed), {wall:.1f} s")
    scf.close()
    m, t = runs["mixed"], runs["fp64_tc"]
    line = {"molecule": f"(H2O){nw}", "basis": "cc-pVDZ", "nbf": srep.nbf, "o": o, "v": v, "frozen_core": False,
            "geometry": f"mpqc_gb300.molecules.water_cluster({nw}, seed=0)", "flops_per_iter": F,
            "e_rhf": e_scf, "scf": {"iters": srep.iters, "eri_s": srep.seconds_eri, "scf_s": srep.seconds_scf,
                                    "one_body_s": srep.seconds_one_body},
            "target_precision": args.solve_precision, "refine_precision": args.refine, "runs": runs}
    if m["s_per_iter_mixed"]:
        line["tflops_mixed"] = F / m["s_per_iter_mixed"] / 1e12
    if t["s_per_iter_fp64"]:
        line["tflops_fp64_tc"] = F / t["s_per_iter_fp64"] / 1e12
    if "fp64" in runs:
        f = runs["fp64"]
        line["abs_dE_mixed_vs_fp64_gpu"] = abs(m["e_corr"] - f["e_corr"])
        line["abs_dE_fp64_tc_vs_fp64_gpu"] = abs(t["e_corr"] - f["e_corr"])
        line["max_abs_dT2_mixed_vs_fp64_gpu"] = float(np.max(np.abs(amps["mixed"] - amps["fp64"])))
        line["max_abs_dT2_fp64_tc_vs_fp64_gpu"] = float(np.max(np.abs(amps["fp64_tc"] - amps["fp64"])))
        if f["s_per_iter_fp64"]:
            line["tflops_fp64"] = F / f["s_per_iter_fp64"] / 1e12
            if m["s_per_iter_mixed"]:
                line["per_iteration_speedup"] = f["s_per_iter_fp64"] / m["s_per_iter_mixed"]
        line["solve_speedup_mixed_vs_fp64"] = f["solve_s"] / m["solve_s"]
        line["solve_speedup_fp64_tc_vs_fp64"] = f["solve_s"] / t["solve_s"]
    if "triples" in m and "triples" in t:
        line["abs_dE_triples_mixed_vs_fp64_tc"] = abs(m["triples"]["e_t"] - t["triples"]["e_t"])
    if ref:
        line["oracle"] = {"e_rhf": ref["e_rhf"], "e_ccsd_corr": ref["e_ccsd_corr"], "source": fixture.name}
        line["abs_dE_rhf_vs_oracle"] = abs(e_scf - ref["e_rhf"])
        for k, r in runs.items():
            line[f"abs_dE_corr_{k}_vs_oracle"] = abs(r["e_corr"] - ref["e_ccsd_corr"])
    print(json.dumps(line), flush=True)
    return 0


def batch_clusters(count, seed):
    """(waters, geometry seed) of each cluster of the batched workload: sizes
    drawn uniformly from 1..6 by the seed, geometries by
    molecules.water_cluster (cube-corner and face-centre sites, random
    orientations, no close contacts)."""
    rng = np.random.default_rng(seed)
    return [(int(n), seed * 1000 + k) for k, n in enumerate(rng.integers(1, 7, size=count))]


def batch_report(args):
    """Batched many-instance CCSD: `--clusters` water clusters (H2O)n, n in
    1..6, in a polarised Pople basis, every cluster's RHF and MO integrals
    built on the GPU, then all mixed-precision solves (split-BF16 bulk
    contractions, FP64 denominators, DIIS, --refine refinement; each stopping at
    its own convergence test) in flight together through gbcc_solve_batch.
    Reports clusters/s of the batch (wall clock of the whole batch per step,
    from t = 0 each step) against the same clusters solved one after another,
    and each cluster's |dE_corr| against its plain-FP64 GPU solve (converged
    to 1e-10)."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    from mpqc_gb300 import build as gb
    gb.build()
    from mpqc_gb300 import RHF, Solver, molecules, solve_batch
    specs = batch_clusters(args.clusters, args.seed)
    t0 = time.perf_counter()
    handles, ref, info = [], [], []
    for n, seed in specs:
        sym, xyz = molecules.water_cluster(n, seed=seed)
        with RHF(sym, xyz, args.batch_basis, threshold=1e-11, max_iter=60) as scf:
            e_scf = scf.run()
            o = scf.nocc()
            v = scf.nbf - o
            s = Solver(o, v, precision="mixed", target_precision=args.solve_precision, max_iter=args.max_iter,
                       refine_iters=2, refine_precision=args.refine, autotune=False)
            scf.ccsd_inputs(s)
            handles.append(s)
            # the plain-FP64 energy of the same MO integrals, tightly converged
            with Solver(o, v, precision="fp64", target_precision=1e-10, max_iter=args.max_iter) as f:
                scf.ccsd_inputs(f)
                ef, _, _, rf = f.solve(want_amplitudes=False)
                ref.append((ef, rf))
        info.append({"waters": n, "seed": seed, "nbf": o + v, "o": o, "v": v, "e_rhf": e_scf})
    prep_s = time.perf_counter() - t0
    log(f"[batch] {len(specs)} clusters, basis {args.batch_basis}, nbf {min(i['nbf'] for i in info)}.."
        f"{max(i['nbf'] for i in info)}: SCF + MO integrals + FP64 solves + handle set-up {prep_s:.1f} s")
    for _ in range(max(1, args.warmup)):  # the first solve of a handle captures its solve graph
        solve_batch(handles)
    walls, res = [], None
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        res = solve_batch(handles)
        walls.append(time.perf_counter() - t1)
    t1 = time.perf_counter()
    seq = [s.solve(want_amplitudes=False) for s in handles]
    seq_s = time.perf_counter() - t1
    for s in handles:
        s.close()
    wall = float(np.median(walls))
    dE = [abs(e - ef) for (e, _), (ef, _) in zip(res, ref)]
    iters = [r.iters for _, r in res]
    line = {"workload": f"{len(specs)} water clusters (H2O)n, n in 1..6 from seed {args.seed}, "
                        f"{args.batch_basis}, mixed-precision CCSD to {args.solve_precision:g}, "
                        f"2 refinement iterations in {args.refine}",
            "metric": "clusters/s (whole batch, from t = 0)", "value": len(specs) / wall, "unit": "clusters/s",
            "steps": len(walls), "ms_per_step": wall * 1e3,
            "sequential_clusters_per_s": len(specs) / seq_s, "batch_speedup_vs_sequential": seq_s / wall,
            "prep_s": prep_s, "all_converged": all(r.converged for _, r in res) and all(r.converged for _, r in ref),
            "iters_min_max": [min(iters), max(iters)],
            "max_abs_dE_mixed_vs_fp64": max(dE), "median_abs_dE_mixed_vs_fp64": float(np.median(dE)),
            "sequential_max_abs_dE_vs_batch": max(abs(a[0] - b[0]) for a, b in zip(seq, res)),
            "nbf_min_max": [min(i["nbf"] for i in info), max(i["nbf"] for i in info)],
            "clusters": [dict(i, e_corr=e, e_corr_fp64=ef, abs_dE=d, iters=r.iters)
                         for i, (e, r), (ef, _), d in zip(info, res, ref, dE)]}
    print(json.dumps(line), flush=True)
    return 0


def triples_probe(args):
    """(T) on seeded synthetic inputs at (--o, --v) (profiling aid): the
    residual-engine handle takes the synthetic integrals, gbcc_triples runs
    twice from the synthetic amplitudes; one JSON line with E(T) and the
    seconds of the second run."""
    from mpqc_gb300 import Solver, synth
    from mpqc_gb300 import build as gb
    gb.build()
    o, v = args.o, args.v
    inp = synth.make_inputs(o, v, 40, seed=args.seed, t1_scale=1e-2)
    ints = {k: np.ascontiguousarray(getattr(inp, k)) for k in
            ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc", "Gabcd")}
    with Solver(o, v, precision="fp64_tc" if args.triples_precision == "fp64_tc" else "fp64") as s:
        s.set_inputs(inp.eps_o, inp.eps_v, **ints)
        s.triples(args.triples_precision, inp.t1, inp.t2)
        t0 = time.perf_counter()
        e_t = s.triples(args.triples_precision, inp.t1, inp.t2)
        sec = time.perf_counter() - t0
    print(json.dumps({"triples": True, "o": o, "v": v, "precision": args.triples_precision, "e_t": e_t,
                      "seconds": sec, "flops_d_terms": 2 * o**3 * v**4}), flush=True)
    return 0


def gemm_probe(args):
    """One GEMM shape C = A B^T on the library's kernels (profiling aid): seeded
    normal FP64 inputs through gbcc_testing_gemm_ex3 (split-BF16 tensor-core
    kernel for --gemm-slices >= 1, plain FP64 for 0); prints one JSON line with
    the kernel time per launch and the executed slice-product TFLOP/s.  The
    launches are what an ncu capture of this command sees
    (``-k regex:gemm_tc_kernel``)."""
    import ctypes as C
    from mpqc_gb300 import _lib, build as gb
    gb.build()
    lib = _lib.load()
    M, N, K = args.gemm
    rng = np.random.default_rng(args.seed)
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K))
    Cm = np.empty((M, N))
    ms = C.c_float()
    sl = args.gemm_slices
    if sl < 0:
        # FP64-grade: six fixed-point slices, 21 pair products in six class launches
        st = lib.gbcc_testing_gemm_fp64tc(M, N, K, A.ctypes.data, B.ctypes.data, Cm.ctypes.data, args.gemm_bn,
                                          args.gemm_ksplit, args.gemm_cta2, args.gemm_repeat, C.byref(ms))
    else:
        st = lib.gbcc_testing_gemm_ex3(M, N, K, A.ctypes.data, B.ctypes.data, Cm.ctypes.data, sl, args.gemm_ksplit,
                                       args.gemm_bn, args.gemm_cta2, args.gemm_chunk, 0, args.gemm_sps,
                                       args.gemm_group, args.gemm_cmode, args.gemm_repeat, C.byref(ms))
    pairs = 21 if sl < 0 else (sl * (sl + 1) // 2 if sl > 0 else 1)
    flops = 2.0 * M * N * K
    out = {"gemm": True, "M": M, "N": N, "K": K, "slices": sl, "bn": args.gemm_bn, "ksplit": args.gemm_ksplit,
           "cta2": args.gemm_cta2, "sps": args.gemm_sps, "group": args.gemm_group, "cmode": args.gemm_cmode,
           "chunk": args.gemm_chunk, "status": st, "ms": ms.value,
           "executed_tflops": pairs * flops / (ms.value * 1e-3) / 1e12 if st == 0 and ms.value > 0 else None,
           "algorithmic_tflops": flops / (ms.value * 1e-3) / 1e12 if st == 0 and ms.value > 0 else None}
    if args.gemm_check and st == 0:
        ref = A @ B.T
        out["max_rel_err"] = float(np.max(np.abs(Cm - ref)) / np.max(np.abs(ref)))
    print(json.dumps(out), flush=True)
    return 0 if st == 0 else 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--o", "--nocc", dest="o", type=int, default=32)
    ap.add_argument("--v", "--nvirt", dest="v", type=int, default=320)
    ap.add_argument("--naux", type=int, default=1200)
    ap.add_argument("--slices", type=int, default=0,
                    help="BF16 slices per operand for every class; 0 (default): chosen per class "
                         "from the measured residual error")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--autotune-table", default=None,
                    help="file of autotuned tiles: loaded if it exists (the contractions it holds are not "
                         "timed again), written after the set-up (profiling runs reuse the plain run's tiles)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default tile per contraction (fewer launches before the first residual)")
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--no-fp64-tc", action="store_true",
                    help="skip the FP64-grade tensor-core residual (and its slice packs)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--residual-only", action="store_true",
                    help="profiling driver: run warmup+steps mixed residuals only")
    ap.add_argument("--solve", action="store_true",
                    help="whole mixed and plain-FP64 solves from t = 0; prints one JSON line")
    ap.add_argument("--b-scale", type=float, default=None,
                    help="std of the DF factor B (default 0.05; with --solve (3e-3 / (v^2 naux))^(1/4))")
    ap.add_argument("--solve-precision", type=float, default=1e-8)
    ap.add_argument("--max-iter", type=int, default=40)
    ap.add_argument("--no-solve-fp64", action="store_true")
    ap.add_argument("--refine", default="fp64_tc", choices=["fp64", "fp64_tc"],
                    help="precision of the refinement iterations of mixed solves (--solve, h2o10, batch64): "
                         "fp64_tc, FP64-grade contractions on the tensor cores (default), or plain FP64")
    ap.add_argument("--cpu-frac", type=float, default=1.0 / 16,
                    help="slab of each contraction's first output index timed by the CPU oracle sample")
    ap.add_argument("--gemm", type=lambda s: tuple(int(x) for x in s.split(",")), default=None,
                    metavar="M,N,K", help="profiling aid: time one GEMM shape on the library's kernels")
    ap.add_argument("--gemm-slices", type=int, default=2,
                    help="BF16 slices (0: plain FP64 kernel; -1: the FP64-grade fixed-point path)")
    ap.add_argument("--gemm-bn", type=int, default=0, help="N tile width (0: the heuristic one)")
    ap.add_argument("--gemm-ksplit", type=int, default=1)
    ap.add_argument("--gemm-cta2", type=int, default=0, help="1: CTA-pair (cta_group::2) variant")
    ap.add_argument("--gemm-chunk", type=int, default=0, help="MMA steps per TMEM accumulation (0: default)")
    ap.add_argument("--gemm-sps", type=int, default=1, help="slices per pipeline stage (2: both slices)")
    ap.add_argument("--gemm-group", type=int, default=1, help="M tiles per band of the tile order (1: rows)")
    ap.add_argument("--gemm-cmode", type=int, default=0,
                    help="output form: bit 0 accumulate into C (beta = 1), bit 1 C unit-stride along M")
    ap.add_argument("--gemm-repeat", type=int, default=5)
    ap.add_argument("--gemm-check", action="store_true",
                    help="also report max |C - A B^T| / max |A B^T| against numpy FP64")
    ap.add_argument("--config", default="residual", choices=["residual", "h2o10", "batch64"],
                    help="residual: the synthetic o=32 v=320 residual (default); h2o10: (H2O)10 / cc-pVDZ "
                         "from the geometry, mixed and plain-FP64 solves against the oracle's energy; "
                         "batch64: 64 water clusters (H2O)1..6 solved together")
    ap.add_argument("--waters", type=int, default=10, help="--config h2o10: cluster size (default 10)")
    ap.add_argument("--triples", action="store_true",
                    help="profiling aid: (T) on synthetic inputs at --o/--v (default 32/320: pass smaller)")
    ap.add_argument("--triples-precision", default="mixed", choices=["fp64", "mixed", "fp64_tc"])
    ap.add_argument("--scf-only", action="store_true", help="--config h2o10: the integrals and RHF only")
    ap.add_argument("--triples-fp64-tc", action="store_true",
                    help="--config h2o10: also the FP64-grade (T) on the fp64_tc solve (mixed (T) always)")
    ap.add_argument("--clusters", type=int, default=64, help="--config batch64: number of clusters")
    ap.add_argument("--batch-basis", default="6-31G**",
                    help="--config batch64: basis (6-31G** gives 25 AO per water; 6-31G* gives 19)")
    args = ap.parse_args()
    if args.gemm:
        return gemm_probe(args)
    if args.triples:
        return triples_probe(args)
    if args.config == "h2o10":
        if args.max_iter == 40 and args.solve_precision == 1e-8:
            args.solve_precision = 1e-9
        return molecule_report(args)
    if args.config == "batch64":
        return batch_report(args)
    if args.impl == "reference":
        return reference_arm(args)
    if args.solve:
        return solve_report(args)
    return ours(args)


if __name__ == "__main__":
    sys.exit(main())
