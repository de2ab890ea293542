"""The C++ client of the C ABI on the GPU (tests/abi_client.cpp): H4/6-31G
from the geometry -- RHF, CCSD through the input producer (mixed) and
through host MO integrals (FP64, host and zero-copy device inputs), the
residual, energy, restarts, (T), a batch and the allocation-free energy --
called as compiled code calls it."""
import os
import subprocess

import pytest

from conftest import build_abi_client

pytestmark = pytest.mark.gpu


def test_cxx_client_end_to_end(tmp_path):
    exe = build_abi_client(tmp_path)
    env = dict(os.environ, GBCC_CLIENT_TMP=str(tmp_path))
    r = subprocess.run([str(exe), "gpu"], capture_output=True, text=True, timeout=600, env=env)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout
