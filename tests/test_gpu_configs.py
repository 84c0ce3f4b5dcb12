"""Parity on the benchmark workloads at their stated sizes (GPU path vs the
CPU oracle, through the C ABI):

  * the small plain-fusion workload exactly: 20 frames 640x480 of the
    4x4x3 m room with 3 spheres, 10 mm voxels, 40 mm truncation, 2^20 hash
    slots, full-volume marching cubes at the end;
  * a later window of the long stream (640x480, 5 mm, 20 mm, 2^22 slots):
    frames 200-204 with per-frame meshes after fusing frames 0-199;
  * every scene of the 64-scene batch (its own extent, voxel size,
    resolution and table), two frames each, compared per scene to the FP64
    oracle;
  * a short run of the HBM-stress workload: 1280x960, 4 mm voxels, 16 mm
    truncation, 2^24 slots, ten frames of the walk through the rooms.

Bar (the integration rule's tolerances): allocated block set and triangle
count bit-exact; with the fp32 oracle every voxel value and every triangle
bit-exact; against the FP64 oracle sdf within 1e-5, weight exact, colour
within one level, and marching cubes of the engine's own volume in FP64
gives the same triangle count with vertices within 1e-4 voxel plus one fp32
ulp of the coordinate.
"""
import numpy as np
import pytest

from helpers import assert_same_blocks, key_set, oracle_for, sort_rows, sorted_blocks, tri_rows
from vhsdf import Batch, Volume, synth

pytestmark = pytest.mark.gpu

SDF_TOL = 1e-5
VERTEX_TOL = 1e-4


def params_for(scene, **kw):
    p = dict(width=scene.width, height=scene.height, fx=scene.fx, fy=scene.fy, cx=scene.cx,
             cy=scene.cy, min_depth=0.1)
    p.update(kw)
    return p


def check_fp64_voxels(g, orc64):
    g = sorted_blocks(g)
    o = sorted_blocks(orc64.export(fp64=True))
    assert np.array_equal(g["xyz"], o["xyz"]), "block set differs from the FP64 oracle's"
    assert np.array_equal(g["weight"].astype(np.float64), o["weight64"])
    err = np.abs(g["sdf"].astype(np.float64) - o["sdf64"])
    assert err.max() <= SDF_TOL * max(1.0, float(np.abs(o["sdf64"]).max()))
    assert np.abs(g["rgb"].astype(int) - o["rgb"].astype(int)).max() <= 1


def check_fp64_mesh(vol, gx, gc, scope="all"):
    """Marching cubes of the engine's own volume by the FP64 oracle: same
    triangle count, vertices within tolerance."""
    e = vol.export_blocks()
    o64 = oracle_for(vol, 64)
    o64.import_blocks(e["xyz"], e["sdf"], e["weight"], e["rgb"])
    if scope == "frame":
        o64.set_frame(vol.block_list())
    m = o64.marching_cubes(scope)
    assert len(gx) == len(m["xyz"])
    a = gx[np.lexsort(tri_rows(gx, gc).T[::-1])].astype(np.float64)
    b = m["xyz64"][np.lexsort(tri_rows(m["xyz"], m["rgb"]).T[::-1])]
    ulp = np.spacing(np.abs(b).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(a - b) <= VERTEX_TOL + ulp)


def check_mesh_fp32(gx, gc, orc32, scope):
    m = orc32.marching_cubes(scope)
    assert len(gx) == len(m["xyz"]) > 0
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))


def test_small_room_at_its_stated_size(gpu):
    """640x480, 10 mm, T = 40 mm, 2^20 slots, 20 frames, final full-volume MC."""
    s = synth.Scene(**synth.SMALL_ROOM)
    assert (s.width, s.height, s.num_frames) == (640, 480, 20)
    vol = Volume(**params_for(s, max_depth=4.0, voxel_size=0.010, trunc=0.040, table_log2=20,
                              pool_blocks=300_000, max_frame_blocks=100_000,
                              max_triangles=4_000_000))
    o32, o64 = oracle_for(vol, 32), oracle_for(vol, 64)
    for f in range(20):
        d, c, p = s.render(f)
        vol.integrate(d, c, p)
        o32.integrate(d, c, p)
        o64.integrate(d, c, p)
        assert key_set(vol.block_list()) == key_set(o32.export(frame=True)["xyz"]), f"frame {f}"
        assert vol.stats()["voxels_updated"] == o32.counts()["voxels_updated"]
    g = vol.export_blocks()
    assert_same_blocks(g, o32.export())
    check_fp64_voxels(g, o64)
    vol.extract("all")
    gx, gc = vol.mesh()
    check_mesh_fp32(gx, gc, o32, "all")
    check_fp64_mesh(vol, gx, gc, "all")


def test_long_stream_later_window(gpu):
    """Frames 200-204 of the long stream after fusing frames 0-199: block
    lists, voxels and per-frame meshes bit-exact with the fp32 oracle."""
    s = synth.Scene(**synth.LONG_STREAM)
    vol = Volume(**params_for(s, max_depth=4.0, voxel_size=0.005, trunc=0.020, table_log2=22,
                              pool_blocks=1_500_000, max_frame_blocks=200_000,
                              max_triangles=8_000_000, flags=0))
    o32 = oracle_for(vol, 32)
    for f in range(200):
        d, c, p = s.render(f)
        vol.integrate(d, c, p)  # asynchronous: frames back to back
        o32.integrate(d, c, p)
    vol.sync()
    for f in range(200, 205):
        d, c, p = s.render(f)
        vol.process_frame(d, c, p)
        o32.integrate(d, c, p)
        vol.sync()
        assert key_set(vol.block_list()) == key_set(o32.export(frame=True)["xyz"]), f"frame {f}"
        gx, gc = vol.mesh()
        check_mesh_fp32(gx, gc, o32, "frame")
    assert_same_blocks(vol.export_blocks(), o32.export())
    gx, gc = vol.mesh()
    check_fp64_mesh(vol, gx, gc, "frame")


def test_every_batched_scene_against_the_fp64_oracle(gpu):
    """The 64 uneven scenes (seeds 100..163: extents 1-8 m, voxels 4-20 mm,
    320x240 .. 1280x960, tables 2^16 .. 2^22) fused together by the batch,
    two frames each; every scene compared with its own FP64 and fp32
    oracles, and its full-volume mesh with the fp32 oracle's."""
    from bench import batch_specs
    specs = batch_specs(64)
    frames = [[sc.render(f) for f in range(2)] for sc, _, _ in specs]
    batch = Batch([dict(prm) for _, _, prm in specs])
    for k in range(2):
        batch.process([fr[k] for fr in frames], with_mesh=False, depth_format="u16")
    status, _ = batch.sync()
    assert all(x == 0 for x in status)
    for i, ((sc, _, prm), fr) in enumerate(zip(specs, frames)):
        vol = batch.scene(i)
        o32, o64 = oracle_for(vol, 32), oracle_for(vol, 64)
        for d, c, p in fr:
            o32.integrate(d, c, p)
            o64.integrate(d, c, p)
        g = vol.export_blocks()
        assert len(g["xyz"]) > 0, f"scene {i}"
        assert_same_blocks(g, o32.export())
        check_fp64_voxels(g, o64)
        vol.extract("all")
        gx, gc = vol.mesh()
        check_mesh_fp32(gx, gc, o32, "all")
    batch.close()


def test_hbm_stress_short_run(gpu):
    """1280x960, 4 mm, T = 16 mm, 2^24 slots: ten frames of the walk (every
    5th of its first 50), fused and extracted; block set, voxels and the
    full-volume mesh bit-exact with the fp32 oracle."""
    s = synth.Scene(kind=4, seed=5, num_frames=2000, width=1280, height=960)
    vol = Volume(**params_for(s, max_depth=4.0, voxel_size=0.004, trunc=0.016, table_log2=24,
                              pool_blocks=600_000, max_frame_blocks=200_000,
                              max_triangles=16_000_000))
    o32 = oracle_for(vol, 32)
    for f in range(0, 50, 5):
        d, c, p = s.render(f)
        vol.integrate(d, c, p)
        o32.integrate(d, c, p)
        assert key_set(vol.block_list()) == key_set(o32.export(frame=True)["xyz"]), f"frame {f}"
    assert_same_blocks(vol.export_blocks(), o32.export())
    vol.extract("all")
    gx, gc = vol.mesh()
    check_mesh_fp32(gx, gc, o32, "all")
