"""Shared helpers of the GPU tests: volumes, oracle twins and comparisons."""
import numpy as np

from oracle.oracle import Oracle
from vhsdf import Volume, synth


def small_scene(w=160, h=120, kind=1, seed=0, frames=20):
    return synth.Scene(kind=kind, seed=seed, num_frames=frames, width=w, height=h)


def volume_for(scene, voxel=0.02, trunc=0.08, max_depth=4.5, **kw):
    params = dict(width=scene.width, height=scene.height, fx=scene.fx, fy=scene.fy,
                  cx=scene.cx, cy=scene.cy, min_depth=0.1, max_depth=max_depth,
                  voxel_size=voxel, trunc=trunc, table_log2=18, pool_blocks=1 << 16,
                  max_frame_blocks=1 << 16, max_triangles=1 << 21)
    params.update(kw)
    return Volume(**params)


def oracle_for(vol, precision=32):
    return Oracle.from_volume_params(vol.params, precision)


def sorted_blocks(e):
    order = np.lexsort(e["xyz"].T[::-1])
    return {k: v[order] for k, v in e.items()}


def key_set(xyz):
    return set(map(tuple, np.asarray(xyz).reshape(-1, 3).tolist()))


def tri_rows(xyz, rgb):
    """Triangles as sortable rows: 9 float bit patterns + 9 colour bytes."""
    fb = np.ascontiguousarray(xyz, np.float32).reshape(-1, 9).view(np.uint32).astype(np.int64)
    return np.concatenate([fb, rgb.reshape(-1, 9).astype(np.int64)], axis=1)


def sort_rows(rows):
    if len(rows) == 0:
        return rows
    return rows[np.lexsort(rows.T[::-1])]


def assert_same_blocks(g, o):
    g, o = sorted_blocks(g), sorted_blocks(o)
    assert np.array_equal(g["xyz"], o["xyz"]), "block sets differ"
    for k in ("sdf", "weight"):
        a = np.ascontiguousarray(g[k]).view(np.uint32)
        b = np.ascontiguousarray(o[k]).view(np.uint32)
        bad = np.argwhere(a != b)
        assert len(bad) == 0, f"{k} differs at {len(bad)} voxels, first {bad[:3].tolist()}"
    assert np.array_equal(g["rgb"], o["rgb"]), "rgb differs"
