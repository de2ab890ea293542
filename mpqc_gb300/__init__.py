"""GB300-native closed-shell CCSD amplitude solver (drop-in for MPQC's CCSD
residual engine and Jacobi/DIIS loop), with its input producer: AO integrals,
RHF and the AO -> MO transform on the GPU.

The compute path is ``libgbcc.so`` (hand-written sm_103a CUDA behind the C
ABI of include/gbcc.h and include/gbcc_scf.h); this package is its host-side
mirror of the reference interface.  Build the library with
``python -m mpqc_gb300.build``.
"""
from . import basis, molecules, synth  # noqa: F401
from ._lib import LIB_PATH, GbccError, load  # noqa: F401
from .ccsd import (CCSD, CCSD_T, FeatureDisabled, InputError, Solver, autotune_clear, autotune_load,  # noqa: F401
                   autotune_save, compute_cs_ccsd_r1_r2, dense_to_tiles, solve_batch, tiles_to_dense)
from .scf import RHF, ccsd_energy  # noqa: F401

__all__ = ["CCSD", "Solver", "compute_cs_ccsd_r1_r2", "GbccError", "InputError", "FeatureDisabled",
           "RHF", "ccsd_energy", "load", "LIB_PATH", "synth", "basis", "molecules", "autotune_save",
           "autotune_load", "autotune_clear", "tiles_to_dense", "dense_to_tiles"]
