"""The synthetic RGB-D generator is deterministic and produces the
reference's input formats."""
import numpy as np

from vhsdf import synth


def test_deterministic_frames():
    a = synth.Scene(kind=2, seed=2, num_frames=500, width=160, height=120)
    b = synth.Scene(kind=2, seed=2, num_frames=500, width=160, height=120)
    assert a.num_objects == b.num_objects == 40
    for f in (0, 123, 499):
        da, ca, pa = a.render(f)
        db, cb, pb = b.render(f)
        assert np.array_equal(da, db) and np.array_equal(ca, cb) and np.array_equal(pa, pb)


def test_formats_and_ranges():
    s = synth.Scene(**synth.SMALL_ROOM)
    d, c, p = s.render(3)
    assert d.dtype == np.uint16 and d.shape == (480, 640)
    assert c.dtype == np.uint8 and c.shape == (480, 640, 3)
    valid = d[d > 0]
    assert valid.min() >= 300 and valid.max() <= 4000
    R = p[:3, :3].astype(np.float64)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-6)
    assert np.allclose(p[3], [0, 0, 0, 1])
    # camera on the 1.5 m circle at 1.4 m height
    assert abs(np.hypot(p[0, 3], p[1, 3]) - 1.5) < 1e-5 and abs(p[2, 3] - 1.4) < 1e-6


def test_noise_is_seeded_and_small():
    s = synth.Scene(**synth.SMALL_ROOM)
    d0, _, _ = s.render(0, noise=False)
    d1, _, _ = s.render(0, noise=True)
    diff = d1.astype(np.int32) - d0.astype(np.int32)
    m = (d0 > 0) & (d1 > 0)
    z = d0[m] / 1000.0
    assert np.std(diff[m] / 1000.0 / (1.5e-3 * z * z)) < 1.5
    assert np.any(diff != 0)


def test_trajectory_speed():
    s = synth.Scene(kind=2, seed=2, num_frames=60, width=64, height=48)
    pos = np.array([s.render(f, noise=False)[2][:3, 3] for f in range(0, 60, 10)])
    step = np.linalg.norm(np.diff(pos, axis=0), axis=1)
    # 0.5 m/s at 30 Hz -> 1/6 m per 10 frames (chord <= arc)
    assert np.all(step <= 1 / 6 + 1e-4) and np.all(step > 0.15)


def test_batched_scene_kinds_vary():
    sizes = set()
    for seed in range(100, 108):
        lo, hi = synth.Scene(kind=3, seed=seed, num_frames=10, width=64, height=48).bounds()
        sizes.add(round(float(hi[0] - lo[0]), 2))
        assert 1.0 <= hi[0] - lo[0] <= 8.0
    assert len(sizes) == 8


def test_multi_room_floor():
    """Kind 4: 20x20x4 m, 4x4 rooms with doors; the camera stays inside the
    floor at 1.5 m, moves at 0.5 m/s and passes from room to room."""
    s = synth.Scene(kind=4, seed=5, num_frames=900, width=80, height=60)
    lo, hi = s.bounds()
    assert np.allclose(lo, [-10, -10, 0]) and np.allclose(hi, [10, 10, 4])
    assert s.num_objects >= 54  # 54 wall pieces (segments and lintels) + objects
    pos = np.array([s.render(f, noise=False)[2][:3, 3] for f in range(0, 900, 30)])
    assert np.all(np.abs(pos[:, :2]) < 10) and np.allclose(pos[:, 2], 1.5, atol=1e-3)
    step = np.linalg.norm(np.diff(pos, axis=0), axis=1)
    assert np.all(step <= 0.5 + 1e-3) and np.all(step > 0.4)  # 30 frames = 0.5 m of arc
    rooms = {(int((x + 10) // 5), int((y + 10) // 5)) for x, y in pos[:, :2]}
    assert len(rooms) >= 3
    d, _, _ = s.render(0)
    assert (d > 0).mean() > 0.5
