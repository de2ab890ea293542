"""Generate the (T) golden fixture: water / 6-31G with cc-pVDZ density
fitting, the inputs of the reference's recorded CCSD(T) run, built by the
oracle (RI-RHF from the Coulomb-metric DF factors, DF MO blocks, CCSD, (T)),
with the energies the reference recorded.

Run in a tree where the reference is present (it reads the geometry and the
recorded energies from there; nothing at test time does):

    python tests/golden/make_ccsd_t.py <MPQC source tree>

Case (reference paths relative to its source tree):

  h2o_ccsd_t_631g   tests/validation/reference/inputs/h2o-ccsd_t-631g-pvdz.json:
                    water (inputs/h2o.xyz), obs 6-31G (13 functions), dfbs
                    cc-pVDZ (24), RI-RHF, CCSD(T) with method df, frozen core
                    (o = 4, v = 8).
                    outputs/h2o-ccsd_t-631g-pvdz.out:233 E_RI-RHF, :336 E_CCSD,
                    :395 E_(T)

The fixture holds the MO blocks built from the DF factors (every block, as
the reference's df method builds them), the active orbital energies, the
oracle's converged T1/T2 and energies, and the recorded energies.  Generation
fails unless the oracle lands within 1e-9 Eh of the recorded RI-RHF and CCSD
energies (the recorded CCSD stopped at dE 2.6e-10) and within 1e-11 Eh of the
recorded (T).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import ccsd_ref as R  # noqa: E402
from oracle import ccsd_t_ref as T  # noqa: E402
from oracle import molecule as M  # noqa: E402

from make_molecules import VALIDATION, recorded  # noqa: E402


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ccsd_t.py <MPQC source tree>")
    ref = Path(sys.argv[1])
    out = ref / VALIDATION / "outputs" / "h2o-ccsd_t-631g-pvdz.out"
    xyz = (ref / VALIDATION / "inputs" / "h2o.xyz").read_text()
    num = r"(-?\d+\.\d+(?:e-?\d+)?)"
    golden = dict(e_rhf=(r"Energy:\s*" + num, 233), e_ccsd=(r"CCSD Energy\s*" + num, 336),
                  e_t=(r"\(T\) Energy:\s*" + num, 395))
    gold = {k: recorded(out, pat, ln) for k, (pat, ln) in golden.items()}
    src = {k: f"{VALIDATION}/outputs/{out.name}:{ln}" for k, (pat, ln) in golden.items()}

    mol = M.Molecule.from_xyz_text(xyz)
    S, H, B = M.df_factors_c(mol, "6-31G", "cc-pVDZ")
    G = np.einsum("kmn,kls->mnls", B, B)
    scf = M.rhf(S, H, G, mol.n_electrons() // 2, mol.nuclear_repulsion())
    nfz = mol.n_frozen_core()
    blocks, eo, ev = M.mo_blocks(scf, G, nfz)
    ora = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=1e-11, max_iter=60)
    e_t = T.triples_energy(ora.t1, ora.t2, blocks["Gijab"], blocks["Gijka"], blocks["Giabc"], eo, ev)
    print(f"RI-RHF {scf.energy:.13f} (recorded {gold['e_rhf']:.13f})")
    print(f"CCSD   {ora.e_corr:.15f} (recorded {gold['e_ccsd']:.15f})")
    print(f"(T)    {e_t:.18f} (recorded {gold['e_t']:.18f})")
    assert abs(scf.energy - gold["e_rhf"]) < 1e-9
    assert ora.converged and abs(ora.e_corr - gold["e_ccsd"]) < 1e-9
    assert abs(e_t - gold["e_t"]) < 1e-11
    # the DF factors in the MO basis (active occupied | virtual), for the
    # density-fitted GPU inputs: Xai[K,a,i] = (K|ai), Xab[K,a,b] = (K|ab)
    C = scf.C
    o = scf.nocc - nfz
    Cocc, Cvir = C[:, nfz:scf.nocc], C[:, scf.nocc:]
    Xai = np.einsum("kmn,ma,ni->kai", B, Cvir, Cocc)
    Xab = np.einsum("kmn,ma,nb->kab", B, Cvir, Cvir)
    np.savez_compressed(
        HERE / "h2o_ccsd_t_631g.npz",
        xyz=xyz, obs="6-31G", dfbs="cc-pVDZ", n_frozen=nfz, o=o, v=ev.size,
        eps_o=eo, eps_v=ev, t1=ora.t1, t2=ora.t2, Xai=Xai, Xab=Xab,
        oracle_e_rhf=scf.energy, oracle_e_ccsd=ora.e_corr, oracle_e_t=e_t,
        ref_e_rhf=gold["e_rhf"], ref_e_ccsd=gold["e_ccsd"], ref_e_t=gold["e_t"],
        ref_sources=np.array([src["e_rhf"], src["e_ccsd"], src["e_t"]]),
        **blocks)


if __name__ == "__main__":
    main()
