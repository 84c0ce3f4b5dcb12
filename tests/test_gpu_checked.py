"""The checked build (per-frame kernels compiled with VH_CHECKED): same
results as the oracle and no failed index check on a normal scene."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_matches_the_oracle(gpu):
    env = dict(os.environ, VHSDF_CHECKED="1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "checked_parity.py")], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "parity ok" in r.stdout
