"""Edge cases of the per-frame path: empty input, bad poses, capacity limits."""
import numpy as np
import pytest

from helpers import oracle_for, small_scene, sort_rows, tri_rows, volume_for
from vhsdf import VhError, _native as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(gpu):
    return small_scene()


def test_empty_depth_changes_nothing(scene):
    vol = volume_for(scene)
    for f in range(3):
        vol.integrate(*scene.render(f))
    before = vol.export_blocks()
    d, c, p = scene.render(5)
    vol.process_frame(np.zeros_like(d), c, p)
    st = vol.stats()
    assert st["frame_blocks"] == 0 and st["voxels_updated"] == 0 and st["triangles"] == 0
    after = vol.export_blocks()
    for k in before:
        assert np.array_equal(before[k], after[k])


def test_non_finite_pose_is_rejected(scene):
    vol = volume_for(scene)
    d, c, p = scene.render(0)
    bad = p.copy()
    bad[0, 3] = np.nan
    with pytest.raises(VhError) as e:
        vol.integrate(d, c, bad)
    assert e.value.status == N.VH_ERR_NOT_FINITE
    vol.integrate(d, c, p)  # still usable
    assert vol.stats()["frames"] == 1


def test_far_away_pose_reports_out_of_range(scene):
    vol = volume_for(scene)
    d, c, p = scene.render(0)
    far = p.copy()
    far[0, 3] = 1.0e6  # 1000 km: beyond the 2^20-block key range at 2 cm voxels
    with pytest.raises(VhError) as e:
        vol.integrate(d, c, far)
    assert e.value.status == N.VH_ERR_OUT_OF_RANGE
    assert vol.stats()["frame_blocks"] == 0


def test_frame_list_capacity(scene):
    vol = volume_for(scene, max_frame_blocks=16)
    with pytest.raises(VhError) as e:
        vol.integrate(*scene.render(0))
    assert e.value.status == N.VH_ERR_CAPACITY


def test_triangle_capacity_per_frame_and_growth(scene):
    vol = volume_for(scene, max_triangles=10)
    orc = oracle_for(vol)
    d, c, p = scene.render(0)
    orc.integrate(d, c, p)
    with pytest.raises(VhError) as e:
        vol.process_frame(d, c, p)
    assert e.value.status == N.VH_ERR_CAPACITY
    # full-volume extraction grows the buffer and matches the oracle
    vol.extract("all")
    gx, gc = vol.mesh()
    m = orc.marching_cubes("all")
    assert len(gx) == len(m["xyz"]) > 10
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))
    # and per-frame extraction now fits too
    vol.process_frame(d, c, p)


def test_bad_arguments(scene):
    vol = volume_for(scene)
    d, c, p = scene.render(0)
    with pytest.raises(TypeError):
        vol.integrate(d.astype(np.int32), c, p)
    L = N.lib()
    assert L.vh_integrate(vol._h, None, 0, None, None, 0) == N.VH_ERR_INVALID_ARG
    assert L.vh_extract(vol._h, 7, None) == N.VH_ERR_INVALID_ARG
    with pytest.raises(VhError) as e:
        vol.render()
    assert e.value.status == N.VH_ERR_UNSUPPORTED


def test_log_callback_sees_handle_and_device_errors(scene):
    """The log callback receives a handle's argument errors with the text
    vh_last_error returns, and a sticky device error (frame-list overflow)
    when the handle reports it."""
    import vhsdf
    got = []
    vhsdf.set_log_callback(lambda level, msg: got.append((level, msg)))
    try:
        vol = volume_for(scene)
        L = N.lib()
        assert L.vh_integrate(vol._h, None, 0, None, None, 0) == N.VH_ERR_INVALID_ARG
        assert got == [(N.VH_LOG_ERROR, L.vh_last_error(vol._h).decode())]
        small = volume_for(scene, max_frame_blocks=16)
        with pytest.raises(VhError):
            small.integrate(*scene.render(0))
        assert len(got) == 2 and got[1][1] == L.vh_last_error(small._h).decode()
    finally:
        vhsdf.set_log_callback(None)


@pytest.mark.parametrize("bad", [2.5, -1.0, np.nan, 2.0 ** 25])
def test_import_rejects_weights_that_are_not_counts(scene, bad):
    """Weights are observation counts (whole numbers); anything else is
    refused before the volume changes."""
    vol = volume_for(scene)
    xyz = np.array([[0, 0, 0], [1, 0, 0]], np.int32)
    sdf = np.zeros((2, 512), np.float32)
    w = np.ones((2, 512), np.float32)
    rgb = np.zeros((2, 512, 3), np.uint8)
    w[1, 17] = bad
    with pytest.raises(VhError) as e:
        vol.import_blocks(xyz, sdf, w, rgb)
    assert e.value.status == N.VH_ERR_INVALID_ARG
    assert len(vol.export_blocks()["xyz"]) == 0
    w[1, 17] = 3.0
    vol.import_blocks(xyz, sdf, w, rgb)
    assert len(vol.export_blocks()["xyz"]) == 2
    vol.close()


def test_reset_clears_volume(scene):
    vol = volume_for(scene)
    vol.integrate(*scene.render(0))
    assert vol.stats()["blocks_allocated"] > 0
    vol.reset()
    st = vol.stats()
    assert st["blocks_allocated"] == 0 and st["frames"] == 0
    assert len(vol.export_blocks()["xyz"]) == 0
    vol.integrate(*scene.render(0))
    orc = oracle_for(vol)
    orc.integrate(*scene.render(0))
    assert vol.stats()["blocks_allocated"] == orc.num_blocks()


def test_external_stream(scene):
    import torch
    vol = volume_for(scene, flags=0)  # asynchronous
    s = torch.cuda.Stream()
    vol.set_stream(s.cuda_stream)
    for f in range(4):
        vol.process_frame(*scene.render(f))
    vol.sync()
    orc = oracle_for(vol)
    for f in range(4):
        orc.integrate(*scene.render(f))
    assert vol.stats()["blocks_allocated"] == orc.num_blocks()


@pytest.mark.parametrize("extra", [0, N.VH_FLAG_DEPTH_FILTER])
def test_pipelined_frames_equal_synchronous_ones(scene, extra):
    """Asynchronous mode, frames submitted back to back: host frames go
    through the two upload slots of the copy stream (pinned buffers, one per
    frame), device frames are read in place (with the depth pre-filter, the
    filter reads them the same way); the volume, the last frame's mesh and
    the counters equal a synchronous run of the same frames."""
    import torch
    from helpers import sorted_blocks
    n = 12
    frames = [scene.render(f) for f in range(n)]
    ref = volume_for(scene, flags=N.VH_FLAG_SYNC | extra)
    for d, c, p in frames:
        ref.process_frame(d, c, p)
    want_st = ref.stats()
    want_tris = sort_rows(tri_rows(*ref.mesh()))
    vol = volume_for(scene, flags=extra)
    fmt = "u16" if frames[0][0].dtype == np.uint16 else "f32"
    signed = np.int16 if fmt == "u16" else np.float32  # torch-friendly view of the bytes
    keep = []
    for f, (d, c, p) in enumerate(frames):
        td, tc = torch.from_numpy(d.view(signed)), torch.from_numpy(c)
        if f % 3 == 2:  # a device frame among host frames
            dd, cc = td.cuda(), tc.cuda()
        else:
            dd, cc = td.pin_memory().numpy().view(d.dtype), tc.pin_memory().numpy()
        keep.append((dd, cc))
        vol.process_frame(dd, cc, p, depth_format=fmt)
    vol.sync()
    st = vol.stats()
    for k in ("frames", "frame_blocks", "blocks_allocated", "voxels_updated", "triangles"):
        assert st[k] == want_st[k], (k, st[k], want_st[k])
    a, b = sorted_blocks(ref.export_blocks()), sorted_blocks(vol.export_blocks())
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(sort_rows(tri_rows(*vol.mesh())), want_tris)
