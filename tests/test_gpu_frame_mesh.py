"""Per-frame meshes delivered to host memory (vh_process_frame_mesh), the
reference's per-frame triangle copy (src/tsdf.cu:1554-1564): every frame's
triangles equal those of vh_process_frame + vh_copy_mesh on a twin volume,
in the synchronous mode and with frames submitted back to back."""
import numpy as np
import pytest

from helpers import small_scene, volume_for
from vhsdf import VhError, _native as N

pytestmark = pytest.mark.gpu


def as_rows(buf, n):
    """(n, 12) float4 triangles -> sorted rows of position bits + colour bits."""
    t = np.ascontiguousarray(buf[:n]).view(np.uint32).astype(np.int64)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


def twin_meshes(scene, frames, **kw):
    vol = volume_for(scene, **kw)
    out = []
    for f in frames:
        vol.process_frame(*scene.render(f))
        n = vol.stats()["triangles"]
        xyz, rgb = vol.mesh()
        out.append((n, xyz, rgb))
    vol.close()
    return out


def rows_from_mesh(xyz, rgb):
    n = len(xyz)
    t = np.zeros((n, 3, 4), np.uint32)
    t[:, :, :3] = np.ascontiguousarray(xyz, np.float32).view(np.uint32)
    c = rgb.astype(np.uint32)
    t[:, :, 3] = c[..., 0] | (c[..., 1] << 8) | (c[..., 2] << 16)
    t = t.reshape(n, 12).astype(np.int64)
    return t[np.lexsort(t.T[::-1])] if n else t


@pytest.mark.parametrize("flags", [N.VH_FLAG_SYNC, 0])
def test_frame_meshes_reach_the_host(gpu, flags):
    scene = small_scene()
    frames = list(range(8))
    ref = twin_meshes(scene, frames)
    vol = volume_for(scene, flags=flags)
    cap = max(n for n, _, _ in ref) + 16
    outs = [np.full((cap, 12), np.nan, np.float32) for _ in frames]
    counts = [np.full(1, -1, np.int64) for _ in frames]
    for f, out, cnt in zip(frames, outs, counts):
        vol.process_frame_mesh(*scene.render(f), out, cnt)
    vol.sync()
    for (n, xyz, rgb), out, cnt in zip(ref, outs, counts):
        assert cnt[0] == n == len(xyz)
        assert np.array_equal(as_rows(out, n), rows_from_mesh(xyz, rgb))
        assert np.all(np.isnan(out[n:]))  # nothing written past the frame's mesh
    # frames 0-6 see the room; frame 7's depth is all invalid (an empty mesh)
    assert all(n > 50_000 for n, _, _ in ref[:7]) and ref[7][0] == 0
    assert vol.stats()["frame_kernels"] == 5


def test_frame_mesh_capacity_is_reported(gpu):
    scene = small_scene()
    vol = volume_for(scene, flags=0)
    out = np.zeros((10, 12), np.float32)
    cnt = np.zeros(1, np.int64)
    vol.process_frame_mesh(*scene.render(0), out, cnt)
    with pytest.raises(VhError) as e:
        vol.sync()
    assert e.value.status == N.VH_ERR_CAPACITY
    assert cnt[0] > 10
    vol.sync()  # reported once


def test_three_buffers_in_turn(gpu):
    """Frames submitted back to back through three host buffers used in
    turn: frame i's mesh is complete once the call for frame i + 2 returns,
    before its buffer is reused by frame i + 3."""
    scene = small_scene(frames=20)
    frames = list(range(12))
    ref = twin_meshes(scene, frames)
    vol = volume_for(scene, flags=0)
    cap = max(n for n, _, _ in ref) + 16
    bufs = [np.zeros((cap, 12), np.float32) for _ in range(3)]
    cnts = [np.zeros(1, np.int64) for _ in range(3)]
    checked = 0

    assert sum(n > 0 for n, _, _ in ref) == 10  # frames 7 and 8 have no valid depth

    def check(i):
        n, xyz, rgb = ref[i]
        assert cnts[i % 3][0] == n
        assert np.array_equal(as_rows(bufs[i % 3], n), rows_from_mesh(xyz, rgb))

    for i, f in enumerate(frames):
        vol.process_frame_mesh(*scene.render(f), bufs[i % 3], cnts[i % 3])
        if i >= 2:
            check(i - 2)
            checked += 1
    vol.sync()
    for i in (len(frames) - 2, len(frames) - 1):
        check(i)
        checked += 1
    assert checked == len(frames)
