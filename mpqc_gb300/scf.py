"""Host-side mirror of MPQC's RHF reference over ``libgbcc`` (include/gbcc_scf.h).

``RHF(kv)`` mirrors the KeyVal constructor of ``lcao::RHF``
(src/mpqc/chemistry/qc/lcao/scf/rhf.h, rhf.cpp:10-44): the molecule (atoms and
Angstrom coordinates, "charge"), the basis name and "max_iter" (30).  The
SCF threshold follows CCSD::evaluate, which converges its reference to
precision / 100 (src/mpqc/chemistry/qc/lcao/cc/ccsd.h:208-211).  Integrals,
Fock builds and the AO -> MO transform run on the GPU; there is no CPU path.

``ccsd_inputs(solver, frozen_core)`` writes the MO integrals and orbital
energies of the standard CCSD method straight into a ``Solver``'s device
inputs, as LCAOFactory::compute4 and make_diagonal_fpq supply them to
CCSD::compute_ccsd in the reference.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from . import basis as B
from . import molecules


@dataclass
class ScfReport:
    nbf: int
    nocc: int
    iters: int
    converged: bool
    energy: float
    e_nuc: float
    seconds_one_body: float
    seconds_eri: float
    seconds_scf: float
    seconds_transform: float


def _scf_check(lib, h, status):
    if status == L.GBCC_OK:
        return status
    msg = lib.gbcc_last_scf_error(h).decode() if h else lib.gbcc_last_scf_error(None).decode()
    raise L.GbccError(status, msg or lib.gbcc_status_string(status).decode())


def n_frozen_core(symbols):
    """Core orbitals that frozen_core freezes (lcao_wfn.h:55: 1s of first-row atoms)."""
    return sum(B.N_CORE[s] for s in symbols)


class RHF:
    """Closed-shell RHF of a molecule on one GPU (one ``gbcc_scf`` handle)."""

    def __init__(self, symbols, coords_angstrom, basis, charge=0, max_iter=30, threshold=1e-11, n_diis=8,
                 device=0, verbose=False):
        self.lib = L.load()
        self.symbols = list(symbols)
        self.basis = basis
        xyz = np.ascontiguousarray(molecules.to_bohr(coords_angstrom), dtype=np.float64)
        zn = np.array([float(B.NUCLEAR_CHARGE[s]) for s in self.symbols])
        atom, ls, nprim, exps, coefs, pure = B.shells_for(self.symbols, basis)
        self._keep = (xyz, zn, atom, ls, nprim, exps, coefs)
        mol = L.Molecule(len(self.symbols), zn.ctypes.data, xyz.ctypes.data, int(charge))
        bas = L.Basis(len(ls), atom.ctypes.data, ls.ctypes.data, nprim.ctypes.data, exps.ctypes.data,
                      coefs.ctypes.data, int(pure))
        cfg = L.ScfConfig()
        self.lib.gbcc_scf_config_default(C.byref(cfg))
        cfg.device, cfg.max_iter, cfg.threshold = int(device), int(max_iter), float(threshold)
        cfg.n_diis, cfg.verbose = int(n_diis), int(bool(verbose))
        h = C.c_void_p()
        _scf_check(self.lib, None, self.lib.gbcc_scf_create(C.byref(h), C.byref(mol), C.byref(bas), C.byref(cfg)))
        self.h = h
        self.report = None
        self.energy = None

    @property
    def nbf(self):
        return B.n_functions(self.symbols, self.basis)

    def run(self):
        rep = L.ScfReport()
        st = self.lib.gbcc_scf_run(self.h, C.byref(rep))
        self.report = ScfReport(rep.nbf, rep.nocc, rep.iters, bool(rep.converged), rep.energy, rep.e_nuc,
                                rep.seconds_one_body, rep.seconds_eri, rep.seconds_scf, rep.seconds_transform)
        _scf_check(self.lib, self.h, st)
        self.energy = rep.energy
        return rep.energy

    def ao(self, eri=False):
        """S, H and (if eri) (mu nu|la si) in the unit-overlap AO basis."""
        n = self.nbf
        S, H = np.empty((n, n)), np.empty((n, n))
        G = np.empty((n, n, n, n)) if eri else None
        _scf_check(self.lib, self.h, self.lib.gbcc_scf_ao(self.h, S.ctypes.data, H.ctypes.data,
                                                          G.ctypes.data if eri else None))
        return S, H, G

    def orbitals(self):
        n = self.nbf
        Cm, eps = np.empty((n, n)), np.empty(n)
        _scf_check(self.lib, self.h, self.lib.gbcc_scf_orbitals(self.h, Cm.ctypes.data, eps.ctypes.data))
        return Cm, eps

    def ccsd_inputs(self, solver, frozen_core=False):
        """Fill and commit ``solver``'s device inputs (o = nocc - n_frozen,
        v = N - nocc) from this reference."""
        nfz = n_frozen_core(self.symbols) if frozen_core else 0
        _scf_check(self.lib, self.h, self.lib.gbcc_scf_ccsd_inputs(self.h, nfz, solver.h))
        return nfz

    def nocc(self, charge=0):
        return (sum(B.NUCLEAR_CHARGE[s] for s in self.symbols) - charge) // 2

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbcc_scf_destroy(self.h)
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


def ccsd_energy(symbols, coords_angstrom, basis, frozen_core=False, charge=0, scf_threshold=1e-11,
                scf_max_iter=60, **solver_kw):
    """RHF -> CCSD of a molecule on the GPU: (E_RHF, E_corr, CCSD report,
    SCF report).  ``solver_kw`` go to ``Solver`` (precision, target_precision,
    max_iter, ...)."""
    from .ccsd import Solver
    with RHF(symbols, coords_angstrom, basis, charge=charge, threshold=scf_threshold,
             max_iter=scf_max_iter, device=solver_kw.get("device", 0)) as scf:
        e_scf = scf.run()
        nocc = scf.nocc(charge)
        nfz = n_frozen_core(symbols) if frozen_core else 0
        o, v = nocc - nfz, scf.nbf - nocc
        with Solver(o, v, **solver_kw) as s:
            scf.ccsd_inputs(s, frozen_core=frozen_core)
            e, _, _, rep = s.solve(want_amplitudes=False)
        return e_scf, e, rep, scf.report
