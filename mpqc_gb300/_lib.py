"""ctypes binding of ``libgbcc.so`` (declarations in include/gbcc.h)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgbcc.so"

GBCC_OK = 0
GBCC_ERR_INVALID_ARG = 1
GBCC_ERR_OOM = 2
GBCC_ERR_CUDA = 3
GBCC_ERR_NOT_CONVERGED = 4
GBCC_ERR_TIMEOUT = 5
GBCC_ERR_STATE = 6
GBCC_ERR_NUMERIC = 7

PREC_FP64 = 0
PREC_MIXED = 1
PREC_FP64_TC = 2

# every symbol include/gbcc.h declares
EXPORTS = (
    "gbcc_abi_version", "gbcc_status_string", "gbcc_config_default", "gbcc_create",
    "gbcc_set_inputs", "gbcc_device_inputs", "gbcc_commit_inputs", "gbcc_residual",
    "gbcc_residual_ex", "gbcc_energy", "gbcc_energy_noalloc", "gbcc_solve", "gbcc_destroy",
    "gbcc_slice_policy", "gbcc_calibrate_slices", "gbcc_last_error", "gbcc_set_amplitudes",
    "gbcc_save_amplitudes", "gbcc_load_amplitudes", "gbcc_set_df_inputs", "gbcc_set_direct_inputs",
    "gbcc_solve_batch", "gbcc_triples", "gbcc_autotune_save", "gbcc_autotune_load", "gbcc_autotune_clear",
    "gbcc_tiles_to_dense", "gbcc_dense_to_tiles",
)
# every symbol include/gbcc_scf.h declares
SCF_EXPORTS = (
    "gbcc_scf_config_default", "gbcc_scf_create", "gbcc_scf_run", "gbcc_scf_ao", "gbcc_scf_orbitals",
    "gbcc_scf_ccsd_inputs", "gbcc_scf_destroy", "gbcc_last_scf_error",
)
# test hooks of include/gbcc_testing.h
TESTING_EXPORTS = ("gbcc_testing_gemm", "gbcc_testing_gemm_ex", "gbcc_testing_gemm_ex2", "gbcc_testing_gemm_ex3", "gbcc_testing_split", "gbcc_testing_scale", "gbcc_testing_fp64_peak", "gbcc_testing_dmma_peak", "gbcc_testing_diis_coefficients", "gbcc_testing_fail_alloc", "gbcc_testing_fixed_split", "gbcc_testing_gemm_fp64tc", "gbcc_testing_gemm_timeout", "gbcc_testing_triples_chunk", "gbcc_testing_profile_residual",
                   "gbcc_testing_last_launches", "gbcc_testing_record", "gbcc_testing_elapsed",
                   "gbcc_testing_profile_gemm_ms", "gbcc_testing_profile_dims",
                   "gbcc_testing_profile_tiles", "gbcc_testing_tc_launches_total", "gbcc_testing_eigh",
                   "gbcc_testing_df_block_rows")


class Config(C.Structure):
    _fields_ = [
        ("o", C.c_int64), ("v", C.c_int64),
        ("precision", C.c_int32), ("slices_ladder", C.c_int32), ("slices_ring", C.c_int32),
        ("slices_other", C.c_int32), ("refine_iters", C.c_int32),
        ("mixed_switch_precision", C.c_double),
        ("max_iter", C.c_int32), ("target_precision", C.c_double),
        ("diis_start", C.c_int32), ("n_diis", C.c_int32), ("diis_damp", C.c_double),
        ("diis_ngroup", C.c_int32), ("diis_group_nstart", C.c_int32),
        ("verbose", C.c_int32), ("device", C.c_int32), ("use_graphs", C.c_int32),
        ("slice_tolerance", C.c_double), ("autotune", C.c_int32), ("refine_reset_diis", C.c_int32),
        ("refine_precision", C.c_int32),
    ]


class Inputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in
                ("eps_o", "eps_v", "Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc", "Gabcd")]


class DfInputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("eps_o", "eps_v", "Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka")] + \
        [("naux", C.c_int64), ("Xai", C.c_void_p), ("Xab", C.c_void_p)]


class DirectInputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("eps_o", "eps_v", "Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka",
                                         "Giabc")] + \
        [("nao", C.c_int64), ("Gao", C.c_void_p), ("Ca", C.c_void_p), ("Ci", C.c_void_p)]


class Report(C.Structure):
    _fields_ = [
        ("iters", C.c_int32), ("converged", C.c_int32), ("mixed_iters", C.c_int32), ("fp64_iters", C.c_int32),
        ("e_corr", C.c_double), ("last_dE", C.c_double), ("last_error", C.c_double),
        ("seconds_total", C.c_double), ("seconds_residual_mixed", C.c_double),
        ("seconds_residual_fp64", C.c_double),
    ]


class Molecule(C.Structure):
    _fields_ = [("natom", C.c_int32), ("charge", C.c_void_p), ("xyz", C.c_void_p), ("mol_charge", C.c_int32)]


class Basis(C.Structure):
    _fields_ = [("nshell", C.c_int32), ("atom", C.c_void_p), ("l", C.c_void_p), ("nprim", C.c_void_p),
                ("exps", C.c_void_p), ("coefs", C.c_void_p), ("pure", C.c_int32)]


class ScfConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_iter", C.c_int32), ("threshold", C.c_double),
                ("n_diis", C.c_int32), ("verbose", C.c_int32)]


class ScfReport(C.Structure):
    _fields_ = [("nbf", C.c_int32), ("nocc", C.c_int32), ("iters", C.c_int32), ("converged", C.c_int32),
                ("energy", C.c_double), ("e_nuc", C.c_double), ("seconds_one_body", C.c_double),
                ("seconds_eri", C.c_double), ("seconds_scf", C.c_double), ("seconds_transform", C.c_double)]


_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the library; raises if it has not been built (there is no
    fallback implementation)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m mpqc_gb300.build` "
                           "(the CUDA extension is required; there is no CPU path)")
    lib = C.CDLL(str(p))
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    lib.gbcc_abi_version.restype = C.c_int
    lib.gbcc_status_string.restype = C.c_char_p
    lib.gbcc_status_string.argtypes = [C.c_int]
    lib.gbcc_config_default.restype = None
    lib.gbcc_config_default.argtypes = [C.POINTER(Config)]
    lib.gbcc_create.restype = C.c_int
    lib.gbcc_create.argtypes = [C.POINTER(vp), C.POINTER(Config)]
    lib.gbcc_set_inputs.restype = C.c_int
    lib.gbcc_set_inputs.argtypes = [vp, C.POINTER(Inputs)]
    lib.gbcc_device_inputs.restype = C.c_int
    lib.gbcc_device_inputs.argtypes = [vp, C.POINTER(Inputs)]
    lib.gbcc_commit_inputs.restype = C.c_int
    lib.gbcc_commit_inputs.argtypes = [vp]
    lib.gbcc_testing_gemm.restype = C.c_int
    lib.gbcc_testing_gemm.argtypes = [C.c_int64, C.c_int64, C.c_int64, vp, vp, vp, C.c_int, C.c_int,
                                      C.POINTER(C.c_float)]
    lib.gbcc_testing_gemm_ex.restype = C.c_int
    lib.gbcc_testing_gemm_ex.argtypes = [C.c_int64, C.c_int64, C.c_int64, vp, vp, vp] + [C.c_int] * 7 + \
        [C.POINTER(C.c_float)]
    lib.gbcc_testing_gemm_ex2.restype = C.c_int
    lib.gbcc_testing_gemm_ex2.argtypes = [C.c_int64, C.c_int64, C.c_int64, vp, vp, vp] + [C.c_int] * 8 + \
        [C.POINTER(C.c_float)]
    lib.gbcc_testing_gemm_ex3.restype = C.c_int
    lib.gbcc_testing_gemm_ex3.argtypes = [C.c_int64, C.c_int64, C.c_int64, vp, vp, vp] + [C.c_int] * 10 + \
        [C.POINTER(C.c_float)]
    lib.gbcc_testing_split.restype = C.c_int
    lib.gbcc_testing_split.argtypes = [vp, C.c_int64, C.c_int, vp]
    lib.gbcc_testing_scale.restype = C.c_int
    lib.gbcc_testing_scale.argtypes = [vp, C.c_int64, C.c_double, vp]
    lib.gbcc_testing_fp64_peak.restype = C.c_int
    lib.gbcc_testing_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    lib.gbcc_testing_dmma_peak.restype = C.c_int
    lib.gbcc_testing_dmma_peak.argtypes = [C.POINTER(C.c_double)]
    lib.gbcc_testing_diis_coefficients.restype = C.c_int
    lib.gbcc_testing_diis_coefficients.argtypes = [C.c_int32, vp, C.c_double, vp, C.POINTER(C.c_int32)]
    lib.gbcc_testing_fail_alloc.restype = C.c_int
    lib.gbcc_testing_fail_alloc.argtypes = [C.c_int64, C.POINTER(C.c_int64)]
    lib.gbcc_testing_triples_chunk.restype = C.c_int
    lib.gbcc_testing_triples_chunk.argtypes = [C.c_int64]
    lib.gbcc_testing_gemm_timeout.restype = C.c_int
    lib.gbcc_testing_gemm_timeout.argtypes = [C.c_int64, C.c_int64, C.c_int64, vp, vp, vp, C.c_uint64, C.c_int64,
                                              C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.gbcc_testing_fixed_split.restype = C.c_int
    lib.gbcc_testing_fixed_split.argtypes = [vp, C.c_int64, C.c_int64, C.c_int, vp, vp]
    lib.gbcc_testing_gemm_fp64tc.restype = C.c_int
    lib.gbcc_testing_gemm_fp64tc.argtypes = [C.c_int64, C.c_int64, C.c_int64, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                             C.c_int, C.POINTER(C.c_float)]
    ip = C.POINTER(C.c_int)
    lib.gbcc_testing_profile_residual.restype = C.c_int
    lib.gbcc_testing_profile_residual.argtypes = [vp, C.c_int, C.c_int, dp, dp, ip, ip, ip]
    lib.gbcc_testing_last_launches.restype = C.c_int
    lib.gbcc_testing_last_launches.argtypes = [vp, ip]
    lib.gbcc_testing_record.restype = C.c_int
    lib.gbcc_testing_record.argtypes = [vp, C.c_int]
    lib.gbcc_testing_elapsed.restype = C.c_int
    lib.gbcc_testing_elapsed.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_float)]
    lib.gbcc_testing_profile_gemm_ms.restype = C.c_int
    lib.gbcc_testing_profile_gemm_ms.argtypes = [vp, C.c_int, dp]
    lib.gbcc_testing_profile_dims.restype = C.c_int
    lib.gbcc_testing_profile_dims.argtypes = [vp, C.c_int, C.POINTER(C.c_int64)]
    lib.gbcc_testing_tc_launches_total.restype = C.c_int
    lib.gbcc_testing_tc_launches_total.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.gbcc_testing_profile_tiles.restype = C.c_int
    lib.gbcc_testing_profile_tiles.argtypes = [vp, C.c_int, C.POINTER(C.c_int32)]
    lib.gbcc_residual.restype = C.c_int
    lib.gbcc_residual.argtypes = [vp, vp, vp, vp, vp]
    lib.gbcc_residual_ex.restype = C.c_int
    lib.gbcc_residual_ex.argtypes = [vp, i32, vp, vp, vp, vp]
    lib.gbcc_energy.restype = C.c_int
    lib.gbcc_energy.argtypes = [vp, vp, vp, vp, vp, dp, dp]
    lib.gbcc_energy_noalloc.restype = C.c_int
    lib.gbcc_energy_noalloc.argtypes = [C.c_int64, C.c_int64, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.gbcc_solve.restype = C.c_int
    lib.gbcc_solve.argtypes = [vp, vp, vp, dp, C.POINTER(Report)]
    lib.gbcc_triples.restype = C.c_int
    lib.gbcc_triples.argtypes = [vp, i32, vp, vp, dp]
    lib.gbcc_solve_batch.restype = C.c_int
    lib.gbcc_solve_batch.argtypes = [C.POINTER(vp), i32, dp, C.POINTER(Report), C.POINTER(C.c_int)]
    lib.gbcc_destroy.restype = C.c_int
    lib.gbcc_destroy.argtypes = [vp]
    lib.gbcc_calibrate_slices.restype = C.c_int
    lib.gbcc_calibrate_slices.argtypes = [vp, vp, vp]
    for name in ("gbcc_autotune_save", "gbcc_autotune_load"):
        getattr(lib, name).restype = C.c_int
        getattr(lib, name).argtypes = [C.c_char_p]
    lib.gbcc_autotune_clear.restype = C.c_int
    lib.gbcc_autotune_clear.argtypes = []
    for name in ("gbcc_tiles_to_dense", "gbcc_dense_to_tiles"):
        getattr(lib, name).restype = C.c_int
        getattr(lib, name).argtypes = [i32, C.POINTER(C.POINTER(C.c_int64)), C.POINTER(C.c_int32), vp, vp]
    lib.gbcc_slice_policy.restype = C.c_int
    lib.gbcc_slice_policy.argtypes = [vp, vp, vp]
    lib.gbcc_last_error.restype = C.c_char_p
    lib.gbcc_last_error.argtypes = [vp]
    lib.gbcc_set_direct_inputs.restype = C.c_int
    lib.gbcc_set_direct_inputs.argtypes = [vp, C.POINTER(DirectInputs)]
    lib.gbcc_set_df_inputs.restype = C.c_int
    lib.gbcc_set_df_inputs.argtypes = [vp, C.POINTER(DfInputs)]
    lib.gbcc_testing_df_block_rows.restype = C.c_int
    lib.gbcc_testing_df_block_rows.argtypes = [C.c_int64]
    lib.gbcc_set_amplitudes.restype = C.c_int
    lib.gbcc_set_amplitudes.argtypes = [vp, vp, vp]
    lib.gbcc_save_amplitudes.restype = C.c_int
    lib.gbcc_save_amplitudes.argtypes = [vp, C.c_char_p]
    lib.gbcc_load_amplitudes.restype = C.c_int
    lib.gbcc_load_amplitudes.argtypes = [vp, C.c_char_p, dp]
    lib.gbcc_scf_config_default.restype = None
    lib.gbcc_scf_config_default.argtypes = [C.POINTER(ScfConfig)]
    lib.gbcc_scf_create.restype = C.c_int
    lib.gbcc_scf_create.argtypes = [C.POINTER(vp), C.POINTER(Molecule), C.POINTER(Basis), C.POINTER(ScfConfig)]
    lib.gbcc_scf_run.restype = C.c_int
    lib.gbcc_scf_run.argtypes = [vp, C.POINTER(ScfReport)]
    lib.gbcc_scf_ao.restype = C.c_int
    lib.gbcc_scf_ao.argtypes = [vp, vp, vp, vp]
    lib.gbcc_scf_orbitals.restype = C.c_int
    lib.gbcc_scf_orbitals.argtypes = [vp, vp, vp]
    lib.gbcc_scf_ccsd_inputs.restype = C.c_int
    lib.gbcc_scf_ccsd_inputs.argtypes = [vp, i32, vp]
    lib.gbcc_scf_destroy.restype = C.c_int
    lib.gbcc_scf_destroy.argtypes = [vp]
    lib.gbcc_last_scf_error.restype = C.c_char_p
    lib.gbcc_last_scf_error.argtypes = [vp]
    lib.gbcc_testing_eigh.restype = C.c_int
    lib.gbcc_testing_eigh.argtypes = [i32, vp, vp, vp]
    del i64
    if path is None:
        _lib = lib
    return lib


class GbccError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gbcc status {status}: {msg}")
        self.status = status
