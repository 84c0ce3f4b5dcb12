"""Parity scenario run against the checked build (VHSDF_CHECKED=1, set by
test_gpu_checked.py before this process imports vhsdf): per-frame fusion and
marching cubes on a small scene and a full-volume extraction, each compared
with the fp32 oracle bit for bit; any failed index check would surface as
VH_ERR_CHECK from the engine.  Exits 0 on success."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (HERE, REPO, os.path.join(REPO, "voxel-hashing-sdf_gb300")):
    sys.path.insert(0, p)

import numpy as np  # noqa: E402

from helpers import (assert_same_blocks, oracle_for, small_scene, sort_rows,  # noqa: E402
                     tri_rows, volume_for)
from vhsdf import _native as N  # noqa: E402


def main():
    assert N.lib().vh_build_flags() & N.VH_BUILD_CHECKED, "not the checked build"
    scene = small_scene()
    for mc_variant in (0, 2):
        vol = volume_for(scene)
        vol.set_tuning(3 if mc_variant else 2, 0, 0, mc_variant)
        orc = oracle_for(vol, 32)
        for f in range(4):
            d, c, p = scene.render(f)
            vol.process_frame(d, c, p)
            orc.integrate(d, c, p)
            gx, gc = vol.mesh()
            m = orc.marching_cubes("frame")
            assert np.array_equal(sort_rows(tri_rows(gx, gc)),
                                  sort_rows(tri_rows(m["xyz"], m["rgb"]))), f
        assert_same_blocks(vol.export_blocks(), orc.export())
        vol.extract("all")
        m = orc.marching_cubes("all")
        assert np.array_equal(sort_rows(tri_rows(*vol.mesh())),
                              sort_rows(tri_rows(m["xyz"], m["rgb"])))
        vol.sync()
        vol.close()
    print("checked build: parity ok")


if __name__ == "__main__":
    main()
