import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) device and the built libgbcc")


def load_golden(name):
    """Fixture inputs rebuilt from the stored DF factor, plus stored outputs."""
    from mpqc_gb300 import synth
    z = np.load(GOLDEN / f"{name}.npz")
    o, v = int(z["o"]), int(z["v"])
    t1 = z["t1"] if "t1" in z else np.zeros((v, o))
    t2 = z["t2"] if "t2" in z else np.zeros((v, v, o, o))
    inp = synth.inputs_from_factor(z["B"], z["eps_o"], z["eps_v"], t1, t2)
    return inp, {k: z[k] for k in z.files}


def ints_dict(inp):
    return {k: np.ascontiguousarray(getattr(inp, k)) for k in
            ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc", "Gabcd")}


def oracle_ints(inp):
    from oracle import ccsd_ref as R
    return R.Integrals(**ints_dict(inp))


def rel_err(x, ref):
    scale = max(float(np.max(np.abs(ref))), 1e-300)
    return float(np.max(np.abs(np.asarray(x) - ref))) / scale


@pytest.fixture(scope="session")
def gbcc_lib():
    """Build (if stale) and load libgbcc; GPU tests only."""
    from mpqc_gb300 import build
    build.build()
    from mpqc_gb300 import _lib
    return _lib.load()


INTEGRAL_NAMES = ("Fia", "Fij", "Fab", "Gijab", "Gijkl", "Giajb", "Gijka", "Giabc", "Gabcd")


def freeze_first_occupied(blocks, eps_o, n=1):
    """Blocks of the same orbitals with the lowest ``n`` occupied orbitals frozen."""
    s = slice(n, None)
    fc = dict(Fia=blocks["Fia"][s], Fij=blocks["Fij"][s, s], Fab=blocks["Fab"],
              Gijab=blocks["Gijab"][s, s], Gijkl=blocks["Gijkl"][s, s, s, s],
              Giajb=blocks["Giajb"][s, :, s], Gijka=blocks["Gijka"][s, s, s],
              Giabc=blocks["Giabc"][s], Gabcd=blocks["Gabcd"])
    return {k: np.ascontiguousarray(v) for k, v in fc.items()}, np.ascontiguousarray(eps_o[s])


def load_molecule(name):
    """Water MO blocks (MPQC annotation order), orbital energies and the whole
    fixture (oracle amplitudes and energies, the reference's recorded energies)."""
    z = np.load(GOLDEN / f"{name}.npz")
    g = {k: z[k] for k in z.files}
    blocks = {k: np.ascontiguousarray(g[k]) for k in INTEGRAL_NAMES}
    return blocks, g["eps_o"], g["eps_v"], g


def build_abi_client(out_dir):
    """Compile tests/abi_client.cpp (a C++ caller of include/gbcc.h and
    gbcc_scf.h) against the in-tree libgbcc.so; returns the executable."""
    import shutil
    import subprocess
    from mpqc_gb300 import _lib, build
    build.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda = Path("/usr/local/cuda")
    lib_dir = Path(_lib.LIB_PATH).resolve().parent
    exe = Path(out_dir) / "abi_client"
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", str(ROOT / "tests" / "abi_client.cpp"), "-I", str(ROOT / "include"),
           "-I", str(cuda / "include"), "-L", str(lib_dir), "-lgbcc", "-L", str(cuda / "lib64"), "-lcudart",
           f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe
