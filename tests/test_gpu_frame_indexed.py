"""Per-frame meshes delivered indexed (vh_process_frame_indexed): expanded
through their faces, every frame's triangles equal the triangle soup of
vh_process_frame_mesh (vertex positions and colours bit for bit), which the
parity tests pin to the oracle; faces number existing vertices only, and
each vertex is shared by several faces."""
import numpy as np
import pytest

from helpers import small_scene, volume_for
from test_gpu_frame_mesh import as_rows, twin_meshes, rows_from_mesh
from vhsdf import VhError, Volume, synth, _native as N

pytestmark = pytest.mark.gpu


def expand(verts, faces, nv, nf):
    """Faces -> (nf, 12) float32 triangles in the soup layout."""
    f = faces[:nf].astype(np.int64)
    assert nf == 0 or (f.min() >= 0 and f.max() < nv), "face numbers a missing vertex"
    return np.ascontiguousarray(verts[:nv][f].reshape(nf, 12))


def run_indexed(vol, scene, frames, vcap, fcap):
    outs = []
    for f in frames:
        v = np.full((vcap, 4), np.nan, np.float32)
        fa = np.full((fcap, 3), -1, np.int32)
        cnt = np.full(2, -1, np.int64)
        vol.process_frame_indexed(*scene.render(f), v, fa, cnt)
        outs.append((v, fa, cnt))
    vol.sync()
    return outs


@pytest.mark.parametrize("flags", [N.VH_FLAG_SYNC, 0])
def test_indexed_meshes_equal_the_triangle_soup(gpu, flags):
    scene = small_scene()
    frames = list(range(8))
    ref = twin_meshes(scene, frames)
    vol = volume_for(scene, flags=flags)
    cap = max(n for n, _, _ in ref) + 16
    outs = run_indexed(vol, scene, frames, cap, cap)
    for (n, xyz, rgb), (v, fa, cnt) in zip(ref, outs):
        nv, nf = int(cnt[0]), int(cnt[1])
        assert nf == n == len(xyz)
        tris = expand(v, fa, nv, nf)
        assert np.array_equal(as_rows(tris, nf), rows_from_mesh(xyz, rgb))
        assert np.all(fa[nf:] == -1) and np.all(np.isnan(v[nv:]))  # nothing past the counts
        if nf:
            assert nv < 1.5 * nf  # shared: a soup has 3 vertices per face
    assert all(n > 50_000 for n, _, _ in ref[:7]) and ref[7][0] == 0
    vol.close()


def test_indexed_and_soup_calls_interleave(gpu):
    """Frames submitted back to back, alternating the two deliveries (they
    share the two device slots and the copy-out stream)."""
    scene = small_scene()
    frames = list(range(6))
    ref = twin_meshes(scene, frames)
    vol = volume_for(scene, flags=0)
    cap = max(n for n, _, _ in ref) + 16
    held = []
    for i, f in enumerate(frames):
        if i % 2:
            out, cnt = np.zeros((cap, 12), np.float32), np.zeros(1, np.int64)
            vol.process_frame_mesh(*scene.render(f), out, cnt)
            held.append(("soup", out, cnt))
        else:
            v, fa, cnt = (np.zeros((cap, 4), np.float32), np.zeros((cap, 3), np.int32),
                          np.zeros(2, np.int64))
            vol.process_frame_indexed(*scene.render(f), v, fa, cnt)
            held.append(("indexed", v, fa, cnt))
    vol.sync()
    for (n, xyz, rgb), h in zip(ref, held):
        if h[0] == "soup":
            assert h[2][0] == n
            got = as_rows(h[1], n)
        else:
            _, v, fa, cnt = h
            assert cnt[1] == n
            got = as_rows(expand(v, fa, int(cnt[0]), n), n)
        assert np.array_equal(got, rows_from_mesh(xyz, rgb))
    vol.close()


def test_indexed_capacity_is_reported(gpu):
    scene = small_scene()
    vol = volume_for(scene, flags=0)
    v, fa, cnt = np.zeros((10, 4), np.float32), np.zeros((10, 3), np.int32), np.zeros(2, np.int64)
    vol.process_frame_indexed(*scene.render(0), v, fa, cnt)
    with pytest.raises(VhError) as e:
        vol.sync()
    assert e.value.status == N.VH_ERR_CAPACITY
    assert cnt[0] > 10 and cnt[1] > 10
    vol.sync()  # reported once
    vol.close()


def test_indexed_meshes_of_the_long_stream(gpu):
    """The benchmark workload (640x480, 5 mm, 2^22 slots): dense noisy
    frames whose blocks exceed one pass's capacities go layer by layer."""
    s = synth.Scene(**synth.LONG_STREAM)
    p = dict(width=640, height=480, fx=s.fx, fy=s.fy, cx=s.cx, cy=s.cy, min_depth=0.1,
             max_depth=4.0, voxel_size=0.005, trunc=0.02, table_log2=22, pool_blocks=400_000,
             max_frame_blocks=200_000, max_triangles=4_000_000)
    soup = Volume(**p)
    idx = Volume(**dict(p, flags=0))
    cap = 4_000_000
    v, fa, cnt = np.zeros((cap, 4), np.float32), np.zeros((cap, 3), np.int32), np.zeros(2, np.int64)
    out, n1 = np.zeros((cap, 12), np.float32), np.zeros(1, np.int64)
    for f in (0, 1, 2, 30):
        frame = s.render(f)
        soup.process_frame_mesh(*frame, out, n1)
        idx.process_frame_indexed(*frame, v, fa, cnt)
        idx.sync()
        nv, nf = int(cnt[0]), int(cnt[1])
        assert nf == n1[0] > 1_000_000
        assert np.array_equal(as_rows(expand(v, fa, nv, nf), nf), as_rows(out, nf))
        assert nv < nf
    soup.close()
    idx.close()
