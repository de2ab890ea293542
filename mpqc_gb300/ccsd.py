"""Host-side mirror of MPQC's closed-shell CCSD interface over ``libgbcc``.

* ``CCSD(kv)`` mirrors the KeyVal constructor of ``lcao::CCSD``
  (src/mpqc/chemistry/qc/lcao/cc/ccsd.h:70-115) and of ``cc::DIISSolver``
  (src/mpqc/chemistry/qc/cc/solvers.h:84-95): same keywords, defaults and
  input errors.  ``compute(integrals)`` replaces ``CCSD::compute_ccsd``
  (ccsd.h:268-477) and returns E_corr; ``t1()`` / ``t2()`` return the
  converged amplitudes as ``CCSD::t1()/t2()`` (ccsd.h:165-179) do.
* ``compute_cs_ccsd_r1_r2(t1, t2, ints)`` evaluates both residuals of
  ccsd_r1_r2.h:70-124 and 198-293 (R1 then R2, as the reference requires).

Arrays are numpy (host) or torch CUDA tensors (device), FP64, C-contiguous,
in MPQC annotation order (t1[a,i], t2[a,b,i,j], Gijab[i,j,a,b], ...).
Every call goes to the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

# precision names: plain FP64 (DFMA), split-BF16 mixed, FP64-grade on the tensor cores
_PRECS = {"fp64": L.PREC_FP64, "mixed": L.PREC_MIXED, "fp64_tc": L.PREC_FP64_TC}

INTEGRAL_NAMES = ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc", "Gabcd")


class InputError(ValueError):
    """Counterpart of mpqc::InputError (src/mpqc/util/core/exception.h)."""


class FeatureDisabled(RuntimeError):
    """Counterpart of mpqc::FeatureDisabled: a reference option this drop-in does not provide."""


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        if x.dtype != np.float64 or not x.flags.c_contiguous:
            raise InputError("arrays must be C-contiguous float64")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):  # torch tensor
        import torch
        if x.dtype != torch.float64 or not x.is_contiguous():
            raise InputError("tensors must be contiguous float64")
        return x.data_ptr()
    raise InputError(f"unsupported array type {type(x)!r}")


def _check(lib, h, status):
    if status in (L.GBCC_OK,):
        return status
    msg = lib.gbcc_last_error(h).decode() if h else lib.gbcc_last_error(None).decode()
    raise L.GbccError(status, msg or lib.gbcc_status_string(status).decode())


@dataclass
class Report:
    iters: int
    converged: bool
    mixed_iters: int
    fp64_iters: int
    e_corr: float
    last_dE: float
    last_error: float
    seconds_total: float
    seconds_residual_mixed: float
    seconds_residual_fp64: float


class Solver:
    """One ``gbcc_handle``: device-resident integrals, residual engine and
    Jacobi+DIIS loop for fixed (o, v)."""

    def __init__(self, o, v, precision="fp64", slices=(0, 0, 0), refine_iters=2,
                 mixed_switch_precision=0.0, max_iter=30, target_precision=1e-9,
                 diis_start=1, n_diis=8, diis_damp=0.0, diis_ngroup=1, diis_group_nstart=1,
                 verbose=False, device=0, use_graphs=2, slice_tolerance=1e-5, autotune=True,
                 refine_reset_diis=True, refine_precision="fp64"):
        self.lib = L.load()
        cfg = L.Config()
        self.lib.gbcc_config_default(C.byref(cfg))
        cfg.o, cfg.v = int(o), int(v)
        cfg.precision = _PRECS[precision]
        cfg.slices_ladder, cfg.slices_ring, cfg.slices_other = (int(s) for s in slices)
        cfg.refine_iters = int(refine_iters)
        cfg.mixed_switch_precision = float(mixed_switch_precision)
        cfg.max_iter = int(max_iter)
        cfg.target_precision = float(target_precision)
        cfg.diis_start, cfg.n_diis = int(diis_start), int(n_diis)
        cfg.diis_damp = float(diis_damp)
        cfg.diis_ngroup, cfg.diis_group_nstart = int(diis_ngroup), int(diis_group_nstart)
        cfg.verbose = int(bool(verbose))
        cfg.device = int(device)
        cfg.use_graphs = int(use_graphs)  # False 0, True 1, or 2 (whole solve as one graph)
        cfg.slice_tolerance = float(slice_tolerance)
        cfg.autotune = int(bool(autotune))
        cfg.refine_reset_diis = int(bool(refine_reset_diis))
        # refinement iterations of a mixed solve: plain FP64 or FP64-grade on the tensor cores
        cfg.refine_precision = _PRECS[refine_precision]
        self.cfg = cfg
        self.o, self.v = int(o), int(v)
        h = C.c_void_p()
        _check(self.lib, None, self.lib.gbcc_create(C.byref(h), C.byref(cfg)))
        self.h = h
        self._keep = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbcc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_inputs(self, eps_o, eps_v, **ints):
        missing = [n for n in INTEGRAL_NAMES if n not in ints]
        if missing:
            raise InputError(f"missing integrals: {missing}")
        inp = L.Inputs()
        inp.eps_o, inp.eps_v = _ptr(eps_o), _ptr(eps_v)
        for n in INTEGRAL_NAMES:
            setattr(inp, n, _ptr(ints[n]))
        self._keep = (eps_o, eps_v, ints)
        _check(self.lib, self.h, self.lib.gbcc_set_inputs(self.h, C.byref(inp)))
        self._keep = None

    def set_df_inputs(self, eps_o, eps_v, Xai, Xab, **ints):
        """Density-fitted inputs (the reference's method "df"): Fia, Fij, Fab,
        Gijab, Gijkl, Giajb, Gijka as for ``set_inputs`` plus the factors
        Xai[K,a,i] = (K|ai) and Xab[K,a,b] = (K|ab); no (ab|cd) array."""
        names = ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka")
        missing = [n for n in names if n not in ints]
        if missing:
            raise InputError(f"missing integrals: {missing}")
        inp = L.DfInputs()
        inp.eps_o, inp.eps_v = _ptr(eps_o), _ptr(eps_v)
        for n in names:
            setattr(inp, n, _ptr(ints[n]))
        inp.naux = int(Xai.shape[0])
        inp.Xai, inp.Xab = _ptr(Xai), _ptr(Xab)
        self._keep = (eps_o, eps_v, Xai, Xab, ints)
        _check(self.lib, self.h, self.lib.gbcc_set_df_inputs(self.h, C.byref(inp)))
        self._keep = None

    def set_direct_inputs(self, eps_o, eps_v, Gao, Ca, Ci, **ints):
        """Integral-direct inputs (the reference's method "direct"): Fia, Fij,
        Fab, Gijab, Gijkl, Giajb, Gijka, Giabc plus the AO integrals
        Gao[p,q,r,s] = (pq|rs) and the MO coefficients Ca[p,a], Ci[p,k]; no
        (ab|cd) array."""
        names = ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc")
        missing = [n for n in names if n not in ints]
        if missing:
            raise InputError(f"missing integrals: {missing}")
        inp = L.DirectInputs()
        inp.eps_o, inp.eps_v = _ptr(eps_o), _ptr(eps_v)
        for n in names:
            setattr(inp, n, _ptr(ints[n]))
        inp.nao = int(Gao.shape[0])
        inp.Gao, inp.Ca, inp.Ci = _ptr(Gao), _ptr(Ca), _ptr(Ci)
        self._keep = (eps_o, eps_v, Gao, Ca, Ci, ints)
        _check(self.lib, self.h, self.lib.gbcc_set_direct_inputs(self.h, C.byref(inp)))
        self._keep = None

    def device_inputs(self):
        """Device pointers (ints) of the handle's own input arrays, to be filled
        on the device before ``commit_inputs()`` (zero-copy set-up)."""
        inp = L.Inputs()
        _check(self.lib, self.h, self.lib.gbcc_device_inputs(self.h, C.byref(inp)))
        return {n: getattr(inp, n) for n in ("eps_o", "eps_v") + INTEGRAL_NAMES}

    def commit_inputs(self):
        _check(self.lib, self.h, self.lib.gbcc_commit_inputs(self.h))

    def profile_residual(self, precision=None, max_sites=256):
        """Per-operation CUDA-event times of one residual on the device-resident
        amplitudes: list of dicts (ms, flops, pairs, cls)."""
        prec = self.cfg.precision if precision is None else _PRECS[precision]
        ms = (C.c_double * max_sites)()
        fl = (C.c_double * max_sites)()
        pr = (C.c_int * max_sites)()
        cl = (C.c_int * max_sites)()
        n = C.c_int()
        _check(self.lib, self.h, self.lib.gbcc_testing_profile_residual(self.h, prec, max_sites, ms, fl, pr, cl,
                                                                        C.byref(n)))
        gm = (C.c_double * max_sites)()
        self.lib.gbcc_testing_profile_gemm_ms(self.h, max_sites, gm)
        mnk = (C.c_int64 * (3 * max_sites))()
        self.lib.gbcc_testing_profile_dims(self.h, max_sites, mnk)
        tl = (C.c_int32 * (4 * max_sites))()
        self.lib.gbcc_testing_profile_tiles(self.h, max_sites, tl)
        return [dict(ms=ms[i], gemm_ms=gm[i], flops=fl[i], pairs=pr[i], cls=cl[i],
                     M=mnk[3 * i], N=mnk[3 * i + 1], K=mnk[3 * i + 2], bn=tl[4 * i], ksplit=tl[4 * i + 1],
                     sps=tl[4 * i + 2], group=tl[4 * i + 3])
                for i in range(min(n.value, max_sites))]

    def tc_launches_total(self):
        n = C.c_int64()
        self.lib.gbcc_testing_tc_launches_total(self.h, C.byref(n))
        return n.value

    def record(self, slot):
        _check(self.lib, self.h, self.lib.gbcc_testing_record(self.h, slot))

    def elapsed_ms(self, slot0, slot1):
        ms = C.c_float()
        _check(self.lib, self.h, self.lib.gbcc_testing_elapsed(self.h, slot0, slot1, C.byref(ms)))
        return ms.value

    def last_launches(self):
        n = C.c_int()
        self.lib.gbcc_testing_last_launches(self.h, C.byref(n))
        return n.value

    def residual(self, t1, t2, r1=None, r2=None, precision=None):
        o, v = self.o, self.v
        if r1 is None:
            r1 = np.empty((v, o)) if isinstance(t1, np.ndarray) else t1.new_empty((v, o))
        if r2 is None:
            r2 = np.empty((v, v, o, o)) if isinstance(t2, np.ndarray) else t2.new_empty((v, v, o, o))
        prec = self.cfg.precision if precision is None else _PRECS[precision]
        _check(self.lib, self.h, self.lib.gbcc_residual_ex(self.h, prec, _ptr(t1), _ptr(t2), _ptr(r1), _ptr(r2)))
        return r1, r2

    def calibrate_slices(self, t1, t2):
        """Re-choose the automatic slice counts at these amplitudes (numpy or
        torch CUDA arrays); returns slice_policy()."""
        _check(self.lib, self.h, self.lib.gbcc_calibrate_slices(self.h, _ptr(t1), _ptr(t2)))
        return self.slice_policy()

    def slice_policy(self):
        """((ladder, ring, other) slice counts in use, measured relative residual
        change of each automatically chosen count against 3 slices or None)."""
        sl = (C.c_int32 * 3)()
        err = (C.c_double * 3)()
        _check(self.lib, self.h, self.lib.gbcc_slice_policy(self.h, sl, err))
        return tuple(sl), tuple(None if e < 0 else e for e in err)

    def energy(self, t1, t2, r1, r2):
        e, err = C.c_double(), C.c_double()
        _check(self.lib, self.h, self.lib.gbcc_energy(self.h, _ptr(t1), _ptr(t2), _ptr(r1), _ptr(r2),
                                                      C.byref(e), C.byref(err)))
        return e.value, err.value

    def set_amplitudes(self, t1, t2):
        """Seed the next ``solve()`` with these amplitudes (a restart; host or device arrays)."""
        self._keep = (t1, t2)
        _check(self.lib, self.h, self.lib.gbcc_set_amplitudes(self.h, _ptr(t1), _ptr(t2)))
        self._keep = None

    def save_amplitudes(self, path):
        """Write the last solve's t1/t2 and energy to a checkpoint file."""
        _check(self.lib, self.h, self.lib.gbcc_save_amplitudes(self.h, str(path).encode()))

    def load_amplitudes(self, path):
        """Seed the next ``solve()`` from a checkpoint; returns its stored energy."""
        e = C.c_double()
        _check(self.lib, self.h, self.lib.gbcc_load_amplitudes(self.h, str(path).encode(), C.byref(e)))
        return e.value

    def triples(self, precision="mixed", t1=None, t2=None):
        """E(T), the perturbative triples correction (``gbcc_triples``; the
        reference's CCSD_T, ccsd_t.h:143-172) from t1/t2 or, when they are
        None, from the amplitudes of the last ``solve()``.  ``precision``
        ("fp64", "mixed", "fp64_tc") sets the arithmetic of the o^3 v^4
        contractions; the energy sums are FP64."""
        e = C.c_double()
        _check(self.lib, self.h, self.lib.gbcc_triples(self.h, _PRECS[precision], _ptr(t1), _ptr(t2), C.byref(e)))
        return e.value

    def solve(self, want_amplitudes=True):
        o, v = self.o, self.v
        t1 = np.empty((v, o)) if want_amplitudes else None
        t2 = np.empty((v, v, o, o)) if want_amplitudes else None
        e = C.c_double()
        rep = L.Report()
        st = self.lib.gbcc_solve(self.h, _ptr(t1), _ptr(t2), C.byref(e), C.byref(rep))
        if st not in (L.GBCC_OK, L.GBCC_ERR_NOT_CONVERGED):
            _check(self.lib, self.h, st)
        r = Report(rep.iters, bool(rep.converged), rep.mixed_iters, rep.fp64_iters, rep.e_corr,
                   rep.last_dE, rep.last_error, rep.seconds_total, rep.seconds_residual_mixed,
                   rep.seconds_residual_fp64)
        return e.value, t1, t2, r


def _report(rep):
    return Report(rep.iters, bool(rep.converged), rep.mixed_iters, rep.fp64_iters, rep.e_corr,
                  rep.last_dE, rep.last_error, rep.seconds_total, rep.seconds_residual_mixed,
                  rep.seconds_residual_fp64)


def autotune_save(path):
    """Write the process's autotune table (tile choices of every tensor-core
    contraction timed so far, by shape) to ``path``."""
    lib = L.load()
    _check(lib, None, lib.gbcc_autotune_save(str(path).encode()))


def autotune_load(path):
    """Merge a table written by autotune_save: handles created afterwards take
    the stored tiles of matching contractions without timing them."""
    lib = L.load()
    _check(lib, None, lib.gbcc_autotune_load(str(path).encode()))


def autotune_clear():
    """Forget every recorded autotune choice of the process."""
    lib = L.load()
    _check(lib, None, lib.gbcc_autotune_clear())


def _tile_bounds(bounds):
    bounds = [np.ascontiguousarray(b, dtype=np.int64) for b in bounds]
    ptrs = (C.POINTER(C.c_int64) * len(bounds))(*[b.ctypes.data_as(C.POINTER(C.c_int64)) for b in bounds])
    counts = (C.c_int32 * len(bounds))(*[b.size for b in bounds])
    return bounds, ptrs, counts


def tiles_to_dense(tiles, bounds):
    """Dense row-major array from a tile-by-tile buffer (TiledArray order:
    tiles row-major over the tile grid, each row-major inside) with boundary
    lists ``bounds`` per dimension, e.g. MPQC's uneven occupied / virtual
    tilings."""
    lib = L.load()
    keep, ptrs, counts = _tile_bounds(bounds)
    tiles = np.ascontiguousarray(tiles, dtype=np.float64)
    dense = np.empty(tuple(int(b[-1]) for b in keep))
    if tiles.size != dense.size:
        raise InputError("tile buffer size does not match the boundaries")
    _check(lib, None, lib.gbcc_tiles_to_dense(len(keep), ptrs, counts, tiles.ctypes.data, dense.ctypes.data))
    return dense


def dense_to_tiles(dense, bounds):
    """The tile-by-tile buffer of a dense array (inverse of tiles_to_dense)."""
    lib = L.load()
    keep, ptrs, counts = _tile_bounds(bounds)
    dense = np.ascontiguousarray(dense, dtype=np.float64)
    if dense.shape != tuple(int(b[-1]) for b in keep):
        raise InputError("array shape does not match the boundaries")
    tiles = np.empty(dense.size)
    _check(lib, None, lib.gbcc_dense_to_tiles(len(keep), ptrs, counts, dense.ctypes.data, tiles.ctypes.data))
    return tiles


def solve_batch(solvers):
    """Solve several independent handles at once (``gbcc_solve_batch``): each
    handle's solve runs on its own stream from its own host thread, so small
    molecules fill the GPU together.  Returns ``[(e_corr, Report), ...]`` in
    input order; the amplitudes stay on the device (``Solver.save_amplitudes``
    reads them back)."""
    solvers = list(solvers)
    if not solvers:
        return []
    lib = solvers[0].lib
    n = len(solvers)
    hs = (C.c_void_p * n)(*[s.h for s in solvers])
    e = (C.c_double * n)()
    reps = (L.Report * n)()
    sts = (C.c_int * n)()
    st = lib.gbcc_solve_batch(hs, n, e, reps, sts)
    if st not in (L.GBCC_OK, L.GBCC_ERR_NOT_CONVERGED):
        bad = next((s for s, k in zip(solvers, sts) if k == st), None)
        _check(lib, bad.h if bad else None, st)
    return [(e[k], _report(reps[k])) for k in range(n)]


def compute_cs_ccsd_r1_r2(t1, t2, ints, eps_o, eps_v, precision="fp64", **kw):
    """R1 and R2 of the standard closed-shell method (ccsd_r1_r2.h:70-124,
    198-293) for one amplitude set; ``ints`` maps the cc::Integrals names
    (Fia ... Gabcd) to arrays."""
    v, o = t1.shape
    with Solver(o, v, precision=precision, **kw) as s:
        s.set_inputs(eps_o, eps_v, **ints)
        return s.residual(t1, t2)


class CCSD:
    """KeyVal-compatible CCSD front end (Jacobi+DIIS solver).

    Recognised keys (reference defaults): ``method`` ("standard"; "df" and
    "direct" as well, whose integrals ``compute`` then takes in their form),
    ``max_iter`` (30), ``solver`` ("jacobi_diis"), ``verbose`` (False),
    ``reduced_abcd_memory`` (True; no effect for the dense standard method),
    ``diis_start`` (1), ``n_diis`` (8), ``diis_damp`` (0.0), ``diis_ngroup`` (1),
    ``diis_group_nstart`` (1), ``precision`` (the Energy property precision,
    1e-9).  Additional keys of this implementation: ``gbcc_precision``
    ("fp64" | "mixed" | "fp64_tc"), ``slices`` ([ladder, ring, other], default [0,0,0]: chosen from the measured
    error), ``refine_iters`` (2), ``refine_precision`` ("fp64" | "fp64_tc"), ``mixed_switch_precision`` (0: the
    target precision), ``device`` (0).
    """

    def __init__(self, kv: dict):
        kv = dict(kv)
        if "ref" not in kv:
            raise InputError("Default Ref in CCSD is not support!")
        method = kv.get("method", "standard")
        if method not in ("standard", "df", "direct", "direct_df"):
            raise InputError(f"invalid method {method!r}")
        if method == "direct_df":
            raise FeatureDisabled("method 'direct_df' is not provided by this solver")
        self.method = method
        solver = kv.get("solver", "jacobi_diis")
        if solver not in ("jacobi_diis", "pno"):
            raise InputError(f"invalid solver {solver!r}")
        if solver != "jacobi_diis":
            raise FeatureDisabled("the PNO solver is not provided by this solver")
        if kv.get("cp_ccsd", False):
            raise FeatureDisabled("CP-CCSD is not provided by this solver")
        self.kv = kv
        self.max_iter = int(kv.get("max_iter", 30))
        self.verbose = bool(kv.get("verbose", False))
        self.precision = float(kv.get("precision", 1e-9))
        self._t1 = self._t2 = None
        self.report = None
        self.energy = None

    def _solver(self, o, v):
        kv = self.kv
        return Solver(o, v, precision=kv.get("gbcc_precision", "fp64"), slices=kv.get("slices", (0, 0, 0)),
                      refine_iters=kv.get("refine_iters", 2), refine_precision=kv.get("refine_precision", "fp64"),
                      mixed_switch_precision=kv.get("mixed_switch_precision", 0.0),
                      max_iter=self.max_iter, target_precision=self.precision,
                      diis_start=kv.get("diis_start", 1), n_diis=kv.get("n_diis", 8),
                      diis_damp=kv.get("diis_damp", 0.0), diis_ngroup=kv.get("diis_ngroup", 1),
                      diis_group_nstart=kv.get("diis_group_nstart", 1), verbose=self.verbose,
                      device=kv.get("device", 0))

    def _set(self, s, eps_o, eps_v, ints):
        """The integrals of the method: standard -- the nine cc::Integrals
        blocks; df -- the seven blocks without Giabc / Gabcd plus the factors
        Xai, Xab; direct -- the eight blocks without Gabcd plus the AO
        integrals Gao and the MO coefficients Ca, Ci."""
        ints = dict(ints)
        if self.method == "df":
            for k in ("Xai", "Xab"):
                if k not in ints:
                    raise InputError(f"method 'df' needs {k}")
            xai, xab = ints.pop("Xai"), ints.pop("Xab")
            s.set_df_inputs(eps_o, eps_v, xai, xab, **{k: x for k, x in ints.items() if k not in ("Giabc", "Gabcd")})
        elif self.method == "direct":
            for k in ("Gao", "Ca", "Ci"):
                if k not in ints:
                    raise InputError(f"method 'direct' needs {k}")
            g, ca, ci = ints.pop("Gao"), ints.pop("Ca"), ints.pop("Ci")
            s.set_direct_inputs(eps_o, eps_v, g, ca, ci, **{k: x for k, x in ints.items() if k != "Gabcd"})
        else:
            s.set_inputs(eps_o, eps_v, **ints)

    def compute(self, eps_o, eps_v, ints) -> float:
        o, v = np.asarray(eps_o).size if isinstance(eps_o, np.ndarray) else eps_o.numel(), \
            np.asarray(eps_v).size if isinstance(eps_v, np.ndarray) else eps_v.numel()
        with self._solver(o, v) as s:
            self._set(s, eps_o, eps_v, ints)
            e, t1, t2, rep = s.solve()
            self._after_solve(s)
        self._t1, self._t2, self.report, self.energy = t1, t2, rep, e
        return e

    def _after_solve(self, s):
        """Hook of subclasses that consume the converged amplitudes on the handle."""

    def t1(self):
        if self._t1 is None:
            raise RuntimeError("CCSD T1 amplitudes have not been computed")
        return self._t1

    def t2(self):
        if self._t2 is None:
            raise RuntimeError("CCSD T2 amplitudes have not been computed")
        return self._t2


class CCSD_T(CCSD):
    """KeyVal-compatible CCSD(T) front end (CCSD_T, ccsd_t.h:33-195): the CCSD
    energy plus the perturbative triples correction of the converged
    amplitudes.  Keys of CCSD plus ``approach`` ("coarse", the reference's
    default, "fine" and "straight" give the same energy -- they differ in how
    the reference distributes the triples over processes -- ; "laplace", a
    quadrature approximation, is not provided), ``reblock_occ`` /
    ``reblock_unocc`` / ``reblock_inner`` (tiling only, accepted and ignored)
    and, of this implementation, ``triples_precision`` ("fp64" | "mixed" |
    "fp64_tc", default "fp64")."""

    def __init__(self, kv: dict):
        super().__init__(kv)
        approach = self.kv.get("approach", "coarse")
        if approach not in ("coarse", "fine", "straight", "laplace"):
            raise InputError(f"invalid approach {approach!r}")
        if approach == "laplace":
            raise FeatureDisabled("the Laplace-transform (T) is not provided by this solver")
        self.triples_energy = None

    def _after_solve(self, s):
        self.triples_energy = s.triples(self.kv.get("triples_precision", "fp64"))

    def compute(self, eps_o, eps_v, ints) -> float:
        e_ccsd = super().compute(eps_o, eps_v, ints)
        self.energy = e_ccsd + self.triples_energy
        return self.energy
