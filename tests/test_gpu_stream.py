"""Out-of-core blocks (vh_stream_out / vh_stream_in): blocks leave HBM for the
handle's host store and come back bit-identical; streaming around a moving
camera with a radius that covers every block a frame can touch gives exactly
the volume and meshes of an unlimited pool."""
import numpy as np
import pytest

from helpers import assert_same_blocks, sort_rows, tri_rows, volume_for
from vhsdf import VhError, synth

pytestmark = pytest.mark.gpu

MAX_DEPTH = 2.0


def room_stream(frames=40, every=10):
    s = synth.Scene(kind=2, seed=2, num_frames=frames * every, width=160, height=120)
    return s, [s.render(f * every) for f in range(frames)]


def make_volume(s, pool):
    return volume_for(s, voxel=0.02, trunc=0.08, max_depth=MAX_DEPTH, table_log2=18,
                      pool_blocks=pool, max_frame_blocks=1 << 15)


def test_round_trip_is_bit_identical(gpu):
    s, frames = room_stream(12)
    vol = make_volume(s, 1 << 16)
    for d, c, p in frames:
        vol.integrate(d, c, p)
    before = vol.export_blocks()
    n = len(before["xyz"])
    assert vol.stream_out([0, 0, 0], 0.0) == n
    assert vol.host_blocks() == n and vol.stats()["blocks_allocated"] == 0
    assert len(vol.export_blocks()["xyz"]) == 0
    assert vol.stream_in([0, 0, 0]) == n and vol.host_blocks() == 0
    assert_same_blocks(vol.export_blocks(), before)


def test_streaming_around_the_camera_equals_an_unlimited_pool(gpu):
    s, frames = room_stream(40)
    # every block a frame touches lies within (max depth + T) x the longest
    # pixel ray (1.25 at 640x480 intrinsics), plus a block for the MC halo
    radius = 1.3 * (MAX_DEPTH + 0.08) + 2 * np.sqrt(3) * 8 * 0.02
    ref = make_volume(s, 1 << 16)
    vol = make_volume(s, 1 << 16)
    peak, meshes_ref, meshes = 0, [], []
    for d, c, p in frames:
        centre = p[:3, 3]
        ref.process_frame(d, c, p)
        meshes_ref.append(sort_rows(tri_rows(*ref.mesh())))
        vol.stream_in(centre, radius)
        vol.process_frame(d, c, p)
        meshes.append(sort_rows(tri_rows(*vol.mesh())))
        vol.stream_out(centre, radius)
        peak = max(peak, vol.stats()["blocks_allocated"] + 0)
    total = ref.stats()["blocks_allocated"]
    assert vol.host_blocks() > 0 and peak < total  # part of the volume lived on the host
    for a, b in zip(meshes, meshes_ref):
        assert np.array_equal(a, b)
    vol.stream_in([0, 0, 0])
    assert_same_blocks(vol.export_blocks(), ref.export_blocks())


def test_stream_in_reports_a_full_pool(gpu):
    """Moving blocks back into a pool that other blocks have filled reports
    VH_ERR_POOL_FULL; the host store keeps the blocks that did not fit."""
    s, frames = room_stream(40)
    far = max(range(len(frames)),
              key=lambda k: np.linalg.norm(frames[k][2][:3, 3] - frames[0][2][:3, 3]))

    def blocks_of(f):
        probe = make_volume(s, 1 << 16)
        probe.integrate(*frames[f])
        return probe.stats()["blocks_allocated"]

    need, need_far = blocks_of(0), blocks_of(far)
    vol = make_volume(s, max(need, need_far) + min(need, need_far) // 4)
    vol.integrate(*frames[0])
    assert vol.stream_out([0, 0, 0], 0.0) == need
    vol.integrate(*frames[far])  # other blocks take most of the pool
    with pytest.raises(VhError) as err:
        vol.stream_in([0, 0, 0])
    assert err.value.status == 4  # VH_ERR_POOL_FULL
    assert vol.host_blocks() == need


def test_repeated_streaming_keeps_the_table_usable(gpu):
    """Every move-out leaves tombstones; a small table stays usable because
    the table is rebuilt once they fill an eighth of it, and the volume
    round-trips unchanged."""
    s, frames = room_stream(6)
    vol = volume_for(s, voxel=0.02, trunc=0.08, max_depth=MAX_DEPTH, table_log2=10,
                     max_probe=256, pool_blocks=1 << 12, max_frame_blocks=1 << 12)
    for d, c, p in frames:
        vol.integrate(d, c, p)
    before = vol.export_blocks()
    n = len(before["xyz"])
    assert n > 40
    for _ in range(12):  # 12 x n erased keys: far more tombstones than slots / 8
        assert vol.stream_out([0, 0, 0], 0.0) == n
        assert vol.stream_in([0, 0, 0]) == n
        assert vol.stats()["tombstones"] <= (1 << 10) // 8 + n
    assert_same_blocks(vol.export_blocks(), before)
    vol.compact_table()
    assert vol.stats()["tombstones"] == 0
    assert_same_blocks(vol.export_blocks(), before)
    vol.integrate(*frames[0])  # integration goes on after a rebuild
