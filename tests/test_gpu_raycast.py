"""Ray casting of the fused surface (vh_raycast) against the FP64 oracle's
march and against the noise-free synthetic depth."""
import numpy as np
import pytest
import torch

from helpers import oracle_for, small_scene, volume_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fused(gpu):
    scene = small_scene(frames=20)
    vol = volume_for(scene)  # 2 cm voxels, 8 cm truncation
    orc = oracle_for(vol, 64)
    for f in range(20):  # the whole camera circle: every view below is fused
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
        orc.integrate(d, c, p)
    return scene, vol, orc


def test_raycast_matches_fp64_march(fused):
    scene, vol, orc = fused
    for f in (3, 8, 14):
        _, _, p = scene.render(f)
        gd, gn, gc = vol.raycast(p)
        od, on = orc.raycast(p)
        gh, oh = gd > 0, od > 0
        assert gh.mean() > 0.9
        assert (gh == oh).mean() > 0.995  # the hit set (silhouettes may differ)
        both = gh & oh
        err = np.abs(gd[both] - od[both])
        assert np.percentile(err, 99) < 1e-4 and np.median(err) < 1e-5
        dots = (gn[both] * on[both]).sum(-1)
        assert np.percentile(dots, 1) > 0.999
        assert np.all(gc[gh].max(-1) > 0)  # hits take the voxel colour


def test_raycast_sees_the_scene(fused):
    scene, vol, orc = fused
    d, _, p = scene.render(12, noise=False)
    gd, gn, _ = vol.raycast(p)
    m = (gd > 0) & (d > 0)
    assert m.mean() > 0.9
    err = np.abs(gd[m] - d[m] * 1e-3)
    assert np.median(err) < 5e-3 and np.percentile(err, 90) < 1.5e-2
    # normals face the camera: n . (camera centre - hit) > 0
    v, u = np.nonzero(m)
    cam = np.stack([(u - scene.cx) / scene.fx, (v - scene.cy) / scene.fy, np.ones_like(u, float)], -1)
    hit = (cam * gd[m][:, None]) @ p[:3, :3].T.astype(np.float64) + p[:3, 3]
    facing = ((p[:3, 3] - hit) * gn[m]).sum(-1)
    assert (facing > 0).mean() > 0.98


def test_raycast_device_buffers_equal_host(fused):
    scene, vol, _ = fused
    _, _, p = scene.render(6)
    hd, hn, hc = vol.raycast(p)
    h, w = hd.shape
    dd = torch.empty((h, w), dtype=torch.float32, device="cuda")
    dn = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    dc = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
    import ctypes as C
    from vhsdf import _native as N
    pose = np.ascontiguousarray(p.astype(np.float32).reshape(16))
    N.check(vol._L.vh_raycast(vol._h, pose.ctypes.data, dd.data_ptr(), dn.data_ptr(),
                              dc.data_ptr(), N.VH_MEM_DEVICE))
    torch.cuda.synchronize()
    assert np.array_equal(dd.cpu().numpy(), hd)
    assert np.array_equal(dn.cpu().numpy(), hn) and np.array_equal(dc.cpu().numpy(), hc)


def test_raycast_empty_volume_misses(gpu):
    scene = small_scene()
    vol = volume_for(scene)
    _, _, p = scene.render(0)
    d, n, c = vol.raycast(p)
    assert not d.any() and not n.any() and not c.any()
