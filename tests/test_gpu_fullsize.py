"""The benchmark workload at full size (640x480, 5 mm voxels, 20 mm
truncation, 2^22 hash slots): size-independent properties plus bit-exact
agreement with the fp32 oracle on the first frames."""
import numpy as np
import pytest

from helpers import assert_same_blocks, key_set, oracle_for, sort_rows, tri_rows
from vhsdf import Volume, synth, _native as N

pytestmark = pytest.mark.gpu

FULL = dict(width=640, height=480, min_depth=0.1, max_depth=4.0, voxel_size=0.005, trunc=0.02,
            table_log2=22, pool_blocks=600_000, max_frame_blocks=200_000,
            max_triangles=8_000_000)


@pytest.fixture(scope="module")
def stream(gpu):
    s = synth.Scene(**synth.LONG_STREAM)
    return s, [s.render(f) for f in range(0, 60, 2)]


def full_volume(s, **kw):
    p = dict(FULL, fx=s.fx, fy=s.fy, cx=s.cx, cy=s.cy)
    p.update(kw)
    return Volume(**p)


def test_first_frames_bit_exact(stream):
    s, frames = stream
    vol = full_volume(s)
    orc = oracle_for(vol, 32)
    for d, c, p in frames[:4]:
        vol.process_frame(d, c, p)
        orc.integrate(d, c, p)
        assert key_set(vol.block_list()) == key_set(orc.export(frame=True)["xyz"])
    assert_same_blocks(vol.export_blocks(), orc.export())
    # per-frame extraction of the last frame
    gx, gc = vol.mesh()
    m = orc.marching_cubes("frame")
    assert len(gx) == len(m["xyz"]) > 100_000
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))


def test_stream_properties(stream):
    s, frames = stream
    vol = full_volume(s)
    total = 0
    for d, c, p in frames:
        vol.process_frame(d, c, p)
        st = vol.stats()
        assert st["device_error"] == 0
        lst = vol.block_list()
        assert len(lst) == st["frame_blocks"] == len(key_set(lst)) > 5000
        assert 0 < st["voxels_updated"] <= st["frame_blocks"] * 512
        total += st["new_blocks"]
    e = vol.export_blocks()
    assert len(e["xyz"]) == total == vol.stats()["blocks_allocated"]
    assert len(key_set(e["xyz"])) == len(e["xyz"])
    w = e["weight"]
    assert w.max() <= len(frames) and np.all(w == np.round(w))
    assert np.all(np.abs(e["sdf"]) <= 1.0)
    # idempotence: an all-invalid frame changes nothing
    d, c, p = frames[-1]
    vol.process_frame(np.zeros_like(d), c, p)
    e2 = vol.export_blocks()
    for k in e:
        assert np.array_equal(e[k], e2[k])


def test_deterministic_across_launch_modes(stream):
    s, frames = stream
    outs = []
    for flags in (N.VH_FLAG_SYNC, N.VH_FLAG_SYNC | N.VH_FLAG_NO_GRAPH):
        vol = full_volume(s, flags=flags)
        for d, c, p in frames[:12]:
            vol.process_frame(d, c, p)
        e = vol.export_blocks()
        order = np.lexsort(e["xyz"].T[::-1])
        outs.append({k: v[order] for k, v in e.items()})
        vol.close()
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k
