"""Reference energies of the (H2O)10 / cc-pVDZ benchmark system from the oracle.

Writes tests/golden/h2o10_ccpvdz.json: the RHF and FP64 CCSD correlation
energies of water_cluster(10, seed=0) (mpqc_gb300/molecules.py: oxygens on the
corners and two face centres of a 2.9 Angstrom cube, random orientations),
cc-pVDZ (240 functions), all electrons correlated (o = 50, v = 190), computed
entirely by the oracle on the CPU: the C restatement of the integrals
(oracle/ints_ref.c), RHF with DIIS, the MO transform and the numpy CCSD
solver converged to 1e-10.  It needs about 45 GB of host memory and an hour
on 8 cores.  Usage: python tests/golden/make_h2o10.py [n_waters]
"""
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mpqc_gb300 import molecules  # noqa: E402
from oracle import ccsd_ref as R  # noqa: E402
from oracle import molecule as M  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 10
    seed, basis, precision = 0, "cc-pVDZ", 1e-10
    sym, xyz = molecules.water_cluster(n, seed=seed)
    mol = M.Molecule(sym, molecules.to_bohr(xyz))
    t0 = time.time()
    S, H, G = M.ao_integrals_c(mol, basis)
    t_ints = time.time() - t0
    print(f"integrals: N = {S.shape[0]}, {t_ints:.0f} s", flush=True)
    nocc = mol.n_electrons() // 2
    scf = M.rhf_lean(S, H, G, nocc, mol.nuclear_repulsion())
    print(f"RHF: {scf.energy:.12f} ({scf.iters} iterations)", flush=True)
    blocks, eo, ev = M.mo_blocks_inplace(scf, G, 0)
    del G
    e_mp2 = M.mp2_energy(blocks, eo, ev)
    print(f"MP2: {e_mp2:.12f}", flush=True)
    t1 = time.time()
    res = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=precision, max_iter=60)
    t_cc = time.time() - t1
    print(f"CCSD: {res.e_corr:.12f} ({res.iters} iterations, converged {res.converged}, {t_cc:.0f} s)", flush=True)
    out = {
        "system": f"(H2O){n}", "generator": f"mpqc_gb300.molecules.water_cluster({n}, seed={seed})",
        "basis": basis, "frozen_core": False, "nbf": int(S.shape[0]), "o": int(len(eo)), "v": int(len(ev)),
        "e_rhf": scf.energy, "e_mp2": e_mp2, "e_ccsd_corr": res.e_corr, "ccsd_iters": res.iters,
        "ccsd_converged": bool(res.converged), "ccsd_target_precision": precision,
        "xyz_angstrom": np.asarray(xyz).round(10).tolist(), "symbols": sym,
        "cpu_seconds": {"integrals": t_ints, "ccsd": t_cc},
        "made_by": "tests/golden/make_h2o10.py (oracle: oracle/ints_ref.c, oracle/molecule.py, oracle/ccsd_ref.py)",
    }
    name = "h2o10_ccpvdz.json" if n == 10 else f"h2o{n}_ccpvdz.json"
    (ROOT / "tests" / "golden" / name).write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", name)


if __name__ == "__main__":
    main()
