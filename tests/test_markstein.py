"""The integration update divides by the truncation T and by the new weight
through correctly rounded reciprocals plus one fused residual correction
(Markstein's theorem); this checks in C that the result is the IEEE
quotient, exhaustively over a stride of all dividends for 12 truncations,
on seeded samples for every weight up to 4096 (the engine uses the table up
to 2048), and on seeded samples of the projection's x / z and y / z.  The GPU parity tests then compare the kernel with the
oracle's IEEE divisions bit for bit."""
import os
import platform
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("markstein") / "markstein_check")
    flags = ["-O2", "-ffp-contract=off"]
    try:  # hardware FMA on x86 when the CPU has it (aarch64 always does)
        if platform.machine() == "x86_64" and " fma " in open("/proc/cpuinfo").read():
            flags.append("-mfma")
    except OSError:
        pass
    subprocess.run([cc] + flags + ["-o", exe, os.path.join(HERE, "markstein_check.c"), "-lm"],
                   check=True)
    return exe


@pytest.mark.parametrize("mode,arg", [(0, 7), (1, 1 << 17), (2, 1 << 29)])
def test_reciprocal_division_is_ieee(checker, mode, arg):
    out = subprocess.run([checker, str(mode), str(arg)], capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stdout
    assert out.stdout.strip().endswith("mismatches 0"), out.stdout
