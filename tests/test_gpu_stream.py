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


def merge_expected(old, new):
    """numpy restatement of the documented merge of two copies of a volume:
    per voxel (a w_a + b w_b) / (w_a + w_b) in float32 (older copy first),
    colour floor((c_a w_a + c_b w_b) / (w_a + w_b)), weights added; a voxel
    seen by one copy keeps that copy's values; keys in one copy only stay."""
    old, new = sort_blocks(old), sort_blocks(new)
    keys = {tuple(k): i for i, k in enumerate(old["xyz"].tolist())}
    out = {k: [] for k in ("xyz", "sdf", "weight", "rgb")}
    seen = set()
    for j, k in enumerate(new["xyz"].tolist()):
        seen.add(tuple(k))
        sdf, w, c = new["sdf"][j].copy(), new["weight"][j].copy(), new["rgb"][j].copy()
        i = keys.get(tuple(k))
        if i is not None:
            os_, ow, oc = old["sdf"][i], old["weight"][i], old["rgb"][i]
            only_old = (w == 0) & (ow > 0)
            both = (w > 0) & (ow > 0)
            wn = (ow + w).astype(np.float32)
            num = (os_ * ow).astype(np.float32) + (sdf * w).astype(np.float32)
            merged = np.divide(num.astype(np.float32), wn, out=np.zeros_like(wn), where=wn > 0)
            csum = oc.astype(np.int64) * ow.astype(np.int64)[:, None] + \
                c.astype(np.int64) * w.astype(np.int64)[:, None]
            cm = (csum // np.maximum(wn, 1).astype(np.int64)[:, None]).astype(np.uint8)
            sdf = np.where(both, merged, np.where(only_old, os_, sdf))
            c = np.where(both[:, None], cm, np.where(only_old[:, None], oc, c))
            w = np.where(both, wn, np.where(only_old, ow, w))
        out["xyz"].append(k)
        out["sdf"].append(sdf)
        out["weight"].append(w)
        out["rgb"].append(c)
    for i, k in enumerate(old["xyz"].tolist()):
        if tuple(k) not in seen:
            out["xyz"].append(k)
            for f in ("sdf", "weight", "rgb"):
                out[f].append(old[f][i])
    return {"xyz": np.array(out["xyz"], np.int32), "sdf": np.array(out["sdf"], np.float32),
            "weight": np.array(out["weight"], np.float32), "rgb": np.array(out["rgb"], np.uint8)}


def sort_blocks(e):
    order = np.lexsort(e["xyz"].T[::-1])
    return {k: v[order] for k, v in e.items()}


@pytest.mark.parametrize("back_by", ["stream_in", "stream_out_then_in"])
def test_recreated_blocks_merge_with_their_stored_copies(gpu, back_by):
    """A frame that reaches moved-out blocks re-creates them; when the stored
    copy meets the resident one again (moved in, or the new one moved out as
    well) the two are merged, so no observation is lost: the result equals
    the merge of the oracle's two partial volumes."""
    from helpers import oracle_for
    s, frames = room_stream(8)
    vol = make_volume(s, 1 << 16)
    first, later = frames[:4], frames[4:]
    for d, c, p in first:
        vol.integrate(d, c, p)
    n = vol.stream_out([0, 0, 0], 0.0)
    assert n > 0 and vol.stats()["blocks_allocated"] == 0
    for d, c, p in later:  # reaches (most of) the moved-out blocks again
        vol.integrate(d, c, p)
    o_old, o_new = oracle_for(vol, 32), oracle_for(vol, 32)
    for d, c, p in first:
        o_old.integrate(d, c, p)
    for d, c, p in later:
        o_new.integrate(d, c, p)
    old, new = o_old.export(), o_new.export()
    both = len(set(map(tuple, old["xyz"].tolist())) & set(map(tuple, new["xyz"].tolist())))
    assert both > n // 2  # the later frames overlap the stored blocks
    if back_by == "stream_out_then_in":
        vol.stream_out([0, 0, 0], 0.0)  # merges on the host store
        assert vol.host_blocks() == len(merge_expected(old, new)["xyz"])
    vol.stream_in([0, 0, 0])
    assert vol.host_blocks() == 0
    assert_same_blocks(vol.export_blocks(), merge_expected(old, new))


def test_async_eviction_round_trip(gpu):
    """vh_evict_async: the blocks leave the volume in stream order and reach
    the host store bit-identical once the copy has finished."""
    s, frames = room_stream(12)
    vol = make_volume(s, 1 << 16)
    for d, c, p in frames:
        vol.integrate(d, c, p)
    before = vol.export_blocks()
    n = len(before["xyz"])
    vol.evict_async([0, 0, 0], 0.0)
    assert vol.stats()["blocks_allocated"] == 0  # gone in stream order
    vol.sync()  # the copy has finished: the blocks are in the store
    assert vol.host_blocks() == n
    assert vol.stream_in([0, 0, 0]) == n
    assert_same_blocks(vol.export_blocks(), before)


def test_async_eviction_around_the_camera_equals_an_unlimited_pool(gpu):
    """Frames submitted back to back (asynchronous mode) with an eviction
    after each frame and the region of the next frame moved back in before
    it: the volume equals an unlimited pool's bit for bit, while part of it
    lived on the host."""
    s, frames = room_stream(40)
    radius = 1.3 * (MAX_DEPTH + 0.08) + 2 * np.sqrt(3) * 8 * 0.02
    ref = make_volume(s, 1 << 16)
    vol = volume_for(s, voxel=0.02, trunc=0.08, max_depth=MAX_DEPTH, table_log2=18,
                     pool_blocks=1 << 16, max_frame_blocks=1 << 15, flags=0)
    stored = 0
    for d, c, p in frames:
        ref.integrate(d, c, p)
        centre = p[:3, 3]
        vol.stream_in(centre, radius)  # waits for the pending evictions
        stored = max(stored, vol.host_blocks())
        vol.integrate(d, c, p)
        vol.evict_async(centre, radius)
    vol.sync()
    assert stored > 0
    vol.stream_in([0, 0, 0])
    assert_same_blocks(vol.export_blocks(), ref.export_blocks())
