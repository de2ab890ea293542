"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports
every symbol include/gbcc.h declares, and rejects bad input with a status
code (no compute calls: there is no GPU on this host)."""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from mpqc_gb300 import build, _lib
    build.build()
    return _lib.load()


def declared_symbols(header="gbcc.h"):
    text = (ROOT / "include" / header).read_text()
    body = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbcc_[a-z0-9_]+)\s*\(", body)))


def test_header_and_binding_agree():
    from mpqc_gb300 import _lib
    assert declared_symbols() == sorted(_lib.EXPORTS)
    assert declared_symbols("gbcc_scf.h") == sorted(_lib.SCF_EXPORTS)
    assert declared_symbols("gbcc_testing.h") == sorted(_lib.TESTING_EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for header in ("gbcc.h", "gbcc_scf.h", "gbcc_testing.h"):
        for name in declared_symbols(header):
            assert hasattr(lib, name), name
    assert lib.gbcc_abi_version() == 6


def test_defaults_follow_the_reference(lib):
    from mpqc_gb300._lib import Config
    c = Config()
    lib.gbcc_config_default(C.byref(c))
    # ccsd.h:104 max_iter 30; cc/solvers.h:93-95 DIIS; energy.h:45 precision 1e-9
    assert c.max_iter == 30 and c.n_diis == 8 and c.diis_start == 1
    assert c.diis_damp == 0.0 and c.diis_ngroup == 1 and c.diis_group_nstart == 1
    assert c.target_precision == 1e-9 and c.precision == 0 and c.use_graphs == 2
    assert (c.slices_ladder, c.slices_ring, c.slices_other) == (0, 0, 0) and c.slice_tolerance == 1e-5
    assert c.mixed_switch_precision == 0.0 and c.autotune == 1 and c.refine_reset_diis == 1
    assert c.refine_precision == 0


@pytest.mark.parametrize("field,value", [("o", 0), ("v", -1), ("n_diis", 0), ("n_diis", 17),
                                         ("slices_ladder", 4), ("slices_ring", -1), ("slice_tolerance", 0.0), ("precision", 7), ("max_iter", 0),
                                         ("target_precision", 0.0), ("diis_damp", -1.0),
                                         ("refine_reset_diis", 2), ("refine_precision", 1),
                                         ("refine_precision", 3), ("precision", 3)])
def test_create_rejects_bad_config(lib, field, value):
    from mpqc_gb300._lib import Config, GBCC_ERR_INVALID_ARG
    c = Config()
    lib.gbcc_config_default(C.byref(c))
    c.o, c.v = 4, 8
    setattr(c, field, value)
    h = C.c_void_p()
    assert lib.gbcc_create(C.byref(h), C.byref(c)) == GBCC_ERR_INVALID_ARG
    assert not h.value
    assert lib.gbcc_last_error(None).decode().startswith("gbcc_create")


def test_null_arguments(lib):
    from mpqc_gb300._lib import GBCC_ERR_INVALID_ARG, GBCC_OK
    assert lib.gbcc_create(None, None) == GBCC_ERR_INVALID_ARG
    assert lib.gbcc_destroy(None) == GBCC_OK
    assert lib.gbcc_residual(None, None, None, None, None) == GBCC_ERR_INVALID_ARG
    assert lib.gbcc_solve(None, None, None, None, None) == GBCC_ERR_INVALID_ARG
    assert lib.gbcc_status_string(4).decode() == "not converged"


def test_create_without_gpu_fails_cleanly(lib):
    from mpqc_gb300._lib import Config, GBCC_ERR_CUDA, GBCC_OK
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c = Config()
    lib.gbcc_config_default(C.byref(c))
    c.o, c.v = 2, 3
    h = C.c_void_p()
    st = lib.gbcc_create(C.byref(h), C.byref(c))
    assert st == GBCC_ERR_CUDA and not h.value
    assert lib.gbcc_last_error(None)


def test_keyval_front_end_validation():
    from mpqc_gb300 import CCSD, FeatureDisabled, InputError
    with pytest.raises(InputError):
        CCSD({})
    with pytest.raises(InputError):
        CCSD({"ref": "scf", "method": "bogus"})
    with pytest.raises(FeatureDisabled):
        CCSD({"ref": "scf", "method": "direct_df"})
    with pytest.raises(FeatureDisabled):
        CCSD({"ref": "scf", "solver": "pno"})
    assert CCSD({"ref": "scf", "method": "df"}).method == "df"
    assert CCSD({"ref": "scf", "method": "direct"}).method == "direct"
    c = CCSD({"ref": "scf"})
    assert c.max_iter == 30 and c.precision == 1e-9
    with pytest.raises(RuntimeError):
        c.t1()
    from mpqc_gb300 import CCSD_T
    with pytest.raises(InputError):
        CCSD_T({"ref": "scf", "approach": "bogus"})
    with pytest.raises(FeatureDisabled):
        CCSD_T({"ref": "scf", "approach": "laplace"})
    assert CCSD_T({"ref": "scf", "approach": "straight"}).triples_energy is None


def test_array_checks():
    from mpqc_gb300.ccsd import _ptr, InputError
    with pytest.raises(InputError):
        _ptr(np.zeros(3, dtype=np.float32))
    with pytest.raises(InputError):
        _ptr(np.zeros((3, 4))[:, ::2])
    assert _ptr(np.zeros(3)) != 0


def test_autotune_table_files(lib, tmp_path):
    """The autotune table's file round trip (no GPU: the table is host state)."""
    from mpqc_gb300._lib import GBCC_ERR_INVALID_ARG, GBCC_OK
    assert lib.gbcc_autotune_clear() == GBCC_OK
    assert lib.gbcc_autotune_load(str(tmp_path / "missing.txt").encode()) == GBCC_ERR_INVALID_ARG
    assert "autotune" in lib.gbcc_last_error(None).decode()
    good = tmp_path / "tune.txt"
    good.write_text("gbcc-autotune 1\n152:c1:10240x10240x10240:s2:n 192 1 0 2 8\n")
    assert lib.gbcc_autotune_load(str(good).encode()) == GBCC_OK
    out = tmp_path / "out.txt"
    assert lib.gbcc_autotune_save(str(out).encode()) == GBCC_OK
    assert out.read_text() == good.read_text()
    for bad in ("gbcc-autotune 2\n", "gbcc-autotune 1\nkey 192 1\n", "gbcc-autotune 1\nkey 300 1 0 1 1\n",
                "gbcc-autotune 1\nkey 64 1 0 3 1\n", "gbcc-autotune 1\nkey 64 1 0 1 1 9\n"):
        f = tmp_path / "bad.txt"
        f.write_text(bad)
        assert lib.gbcc_autotune_load(str(f).encode()) == GBCC_ERR_INVALID_ARG, bad
    assert lib.gbcc_autotune_save(str(out).encode()) == GBCC_OK
    assert out.read_text() == good.read_text()  # a rejected file leaves the table unchanged
    assert lib.gbcc_autotune_save(str(tmp_path / "no" / "dir.txt").encode()) == GBCC_ERR_INVALID_ARG
    assert lib.gbcc_autotune_clear() == GBCC_OK
    assert lib.gbcc_autotune_save(str(out).encode()) == GBCC_OK
    assert out.read_text() == "gbcc-autotune 1\n"


def test_cxx_client_error_paths(lib, tmp_path):
    """tests/abi_client.cpp, compiled against the headers and libgbcc.so,
    calls every entry point and checks the status each reports without a GPU."""
    import subprocess
    import torch
    from conftest import build_abi_client
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the gpu test runs the client's device flow)")
    exe = build_abi_client(tmp_path)
    r = subprocess.run([str(exe), "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout


def _uneven_bounds(rng, extent, lo, hi):
    """TiledRange1-style boundaries with tile sizes drawn in [lo, hi] (the last one
    takes the remainder)."""
    b = [0]
    while b[-1] < extent:
        b.append(min(extent, b[-1] + int(rng.integers(lo, hi + 1))))
    return np.array(b, dtype=np.int64)


def _tiles_np(dense, bounds):
    """Restatement of the tile-by-tile order: tiles row-major over the grid,
    each one row-major inside."""
    import itertools
    out = []
    for idx in itertools.product(*[range(len(b) - 1) for b in bounds]):
        sl = tuple(slice(b[i], b[i + 1]) for b, i in zip(bounds, idx))
        out.append(dense[sl].ravel())
    return np.concatenate(out)


@pytest.mark.parametrize("shape,lo,hi", [((7,), 1, 3), ((5, 9), 2, 4), ((3, 4, 6, 7), 1, 3), ((6, 6, 5, 5), 2, 3),
                                         ((2, 3, 2, 3, 2), 1, 2)])
def test_tile_layout_adapters(lib, shape, lo, hi):
    """TiledArray-style tiled buffers <-> the dense arrays the entry points take
    (uneven tiles, as MPQC's occupied and virtual tilings are), against numpy."""
    from mpqc_gb300 import dense_to_tiles, tiles_to_dense
    rng = np.random.default_rng(len(shape) * 10 + sum(shape))
    bounds = [_uneven_bounds(rng, n, lo, hi) for n in shape]
    dense = rng.normal(size=shape)
    tiles = _tiles_np(dense, bounds)
    assert np.array_equal(dense_to_tiles(dense, bounds), tiles)
    assert np.array_equal(tiles_to_dense(tiles, bounds), dense)


def test_tile_layout_adapters_reject_bad_bounds(lib):
    import ctypes as C
    from mpqc_gb300 import InputError, tiles_to_dense
    from mpqc_gb300._lib import GbccError
    for bad in ([np.array([1, 3])], [np.array([0, 2, 2])], [np.array([0])]):
        with pytest.raises(GbccError):
            tiles_to_dense(np.zeros(int(bad[0][-1])), bad)
    with pytest.raises(InputError):
        tiles_to_dense(np.zeros(5), [np.array([0, 2, 4])])
    assert lib.gbcc_tiles_to_dense(0, None, None, None, None) == 1
    assert lib.gbcc_dense_to_tiles(9, None, None, None, None) == 1
    assert "rank" in lib.gbcc_last_error(None).decode()
    b = np.array([0, 2], dtype=np.int64)
    ptrs = (C.POINTER(C.c_int64) * 1)(b.ctypes.data_as(C.POINTER(C.c_int64)))
    n = (C.c_int32 * 1)(2)
    assert lib.gbcc_tiles_to_dense(1, ptrs, n, None, None) == 1


def test_energy_noalloc_rejects_sizes_beyond_its_scratch(lib):
    from mpqc_gb300._lib import GBCC_ERR_INVALID_ARG
    st = lib.gbcc_energy_noalloc(4, 513, None, None, None, None, None, None, None, None)
    assert st == GBCC_ERR_INVALID_ARG
    assert "v <= 512" in lib.gbcc_last_error(None).decode()
    assert lib.gbcc_energy_noalloc(0, 8, None, None, None, None, None, None, None, None) == GBCC_ERR_INVALID_ARG
