"""The integer colour average of the integration kernel (weights up to 2048)
is exact under the reciprocal's documented error: an exhaustive check in C
(about 1e9 cases, a few seconds)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_umulhi_floor_division_is_exact(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "blend_bound_check")
    subprocess.run([cc, "-O2", "-o", exe, os.path.join(HERE, "blend_bound_check.c"), "-lm"],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert out.stdout.strip().endswith("failures 0"), out.stdout
