"""Regenerates tests/golden/ref_golden.json from the reference's own code.

Builds oracle/ref_golden (the reference's unmodified src/tsdf.cu plus a
host-side driver, outputs under oracle/_ref/) and runs it on the CPU.  Needs
the reference checkout named by $VH_REFERENCE; the committed
JSON is what the tests read, so the tests themselves never need the reference.

    VH_REFERENCE=<reference checkout> python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("VH_REFERENCE", "")


def build_and_run():
    mk = os.path.join(REPO, "oracle", "ref_golden")
    subprocess.run(["make", "-C", mk, f"REF={REF}", "-j2"], check=True)
    exe = os.path.join(REPO, "oracle", "_ref", "ref_golden")
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120)
    return json.loads(out.stdout)


def main():
    if not REF or not os.path.isdir(REF):
        print("set VH_REFERENCE to the reference checkout", file=sys.stderr)
        return 1
    data = build_and_run()
    data["_source"] = ("outputs of the reference's host code (include/tsdf.cuh, "
                       "include/vhashing.h, src/tsdf.cu) run by oracle/ref_golden; "
                       "floats are IEEE-754 bit patterns")
    path = os.path.join(HERE, "ref_golden.json")
    with open(path, "w") as f:
        json.dump(data, f, separators=(",", ":"))
    print(f"wrote {path}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
