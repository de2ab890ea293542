"""Generate the molecular golden fixtures: water MO integrals from the oracle's
own integral + RHF code, with the energies the reference recorded for the same
inputs in its validation outputs.

Run in a tree where the reference is present (it reads the geometry and the
recorded energies from there; nothing at test time does):

    python tests/golden/make_molecules.py [reference_root]

Cases (reference paths relative to its source tree):

  h2o_631g      tests/validation/reference/inputs/h2o-ccsd-direct-631g.json
                water (inputs/h2o.xyz), 6-31G, 13 functions, frozen core
                (o = 4, v = 8), precision 1e-11.
                outputs/h2o-ccsd-direct-631g.out:228 E_RHF, :280 E_MP2, :304 E_CCSD,
                :291-303 the iteration table (from MP2 amplitudes)
  h2o_ccpvdz    inputs/h2o-eom-ip-ccsd-pvdz.json: same geometry, cc-pVDZ (24
                functions), method standard, frozen_core false (o = 5, v = 19),
                precision 1e-9.
                outputs/h2o-eom-ip-ccsd-pvdz.out:219 E_RHF, :266 E_CCSD
                and, from the same orbitals with the O 1s frozen (o = 4),
                outputs/h2o-eom-ea-ccsd-pvdz.out:265 E_CCSD (frozen_core default true)

Each fixture holds the geometry, the MO blocks in MPQC annotation order, the
active orbital energies, the oracle's converged T1/T2 and energies, and the
reference's recorded energies.  Generation fails unless every oracle energy is
within 1e-9 Eh (check.py's default Energy precision) of the recorded one.
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import ccsd_ref as R  # noqa: E402
from oracle import molecule as M  # noqa: E402

VALIDATION = "tests/validation/reference"


def recorded(path, pattern, line_no):
    lines = Path(path).read_text().splitlines()
    m = re.search(pattern, lines[line_no - 1])
    assert m, (path, line_no, lines[line_no - 1])
    return float(m.group(1))


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_molecules.py <MPQC source tree>")
    ref = Path(sys.argv[1])
    out = ref / VALIDATION / "outputs"
    xyz = (ref / VALIDATION / "inputs" / "h2o.xyz").read_text()
    num = r"(-?\d+\.\d+(?:e-?\d+)?)"

    cases = {
        "h2o_631g": dict(
            basis="6-31G", frozen_core=True, precision=1e-11,
            golden=dict(
                e_rhf=(out / "h2o-ccsd-direct-631g.out", r"Energy:\s*" + num, 228),
                e_mp2=(out / "h2o-ccsd-direct-631g.out", r"MP2 Energy\s*" + num, 280),
                e_ccsd=(out / "h2o-ccsd-direct-631g.out", r"CCSD Energy\s*" + num, 304),
            )),
        "h2o_ccpvdz": dict(
            basis="cc-pVDZ", frozen_core=False, precision=1e-9,
            golden=dict(
                e_rhf=(out / "h2o-eom-ip-ccsd-pvdz.out", r"Energy:\s*" + num, 219),
                e_ccsd=(out / "h2o-eom-ip-ccsd-pvdz.out", r"CCSD Energy\s*" + num, 266),
                e_ccsd_fc=(out / "h2o-eom-ea-ccsd-pvdz.out", r"CCSD Energy\s*" + num, 265),
            )),
    }
    for name, c in cases.items():
        scf, blocks, eo, ev, nfz = M.molecular_inputs(xyz, c["basis"], frozen_core=c["frozen_core"])
        gold = {k: recorded(p, pat, ln) for k, (p, pat, ln) in c["golden"].items()}
        src = {k: f"{VALIDATION}/outputs/{p.name}:{ln}" for k, (p, pat, ln) in c["golden"].items()}
        res = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=1e-11, max_iter=60)
        ours = dict(e_rhf=scf.energy, e_ccsd=res.e_corr, e_mp2=M.mp2_energy(blocks, eo, ev))
        if "e_ccsd_fc" in gold:
            fc = dict(Fia=blocks["Fia"][1:], Fij=blocks["Fij"][1:, 1:], Fab=blocks["Fab"],
                      Gijab=blocks["Gijab"][1:, 1:], Gijkl=blocks["Gijkl"][1:, 1:, 1:, 1:],
                      Giajb=blocks["Giajb"][1:, :, 1:], Gijka=blocks["Gijka"][1:, 1:, 1:],
                      Giabc=blocks["Giabc"][1:], Gabcd=blocks["Gabcd"])
            rfc = R.solve_ccsd(R.Integrals(**fc), eo[1:], ev, target_precision=1e-11, max_iter=60)
            ours["e_ccsd_fc"] = rfc.e_corr
        for k, g in gold.items():
            d = abs(ours[k] - g)
            print(f"{name:12s} {k:10s} ours {ours[k]: .15f} recorded {g: .15f} |d| {d:.1e}")
            assert d <= 1e-9, (name, k)
        extra = {}
        if name == "h2o_631g":
            # the recorded iteration table (iter, deltaE, residual, energy, ...) of a
            # build that started from MP2 amplitudes
            lines = (out / "h2o-ccsd-direct-631g.out").read_text().splitlines()[290:303]
            rows = [[float(x) for x in ln.split()[:4]] for ln in lines]
            assert [int(r[0]) for r in rows] == list(range(13)), lines
            extra["ref_trace"] = np.array([r[1:4] for r in rows])
            extra["ref_trace_source"] = np.array(f"{VALIDATION}/outputs/h2o-ccsd-direct-631g.out:291-303")
            mp2 = R.solve_ccsd(R.Integrals(**blocks), eo, ev, target_precision=1e-11, max_iter=60,
                               initial="mp2")
            worst = max(abs(h[3] - r[2]) for h, r in zip(mp2.history, extra["ref_trace"]))
            print(f"{name:12s} MP2-start trace: max |E - recorded| over 13 rows {worst:.1e}")
            assert worst < 6e-13
        np.savez_compressed(
            HERE / f"{name}.npz",
            xyz=np.array(xyz), basis=np.array(c["basis"]), frozen_core=np.array(c["frozen_core"]),
            n_frozen=np.array(nfz), precision=np.array(c["precision"]),
            eps_o=eo, eps_v=ev, t1=res.t1, t2=res.t2,
            **blocks,
            **{f"oracle_{k}": np.array(v) for k, v in ours.items()},
            **{f"ref_{k}": np.array(v) for k, v in gold.items()},
            **{f"ref_{k}_source": np.array(v) for k, v in src.items()},
            **extra,
        )


if __name__ == "__main__":
    main()
