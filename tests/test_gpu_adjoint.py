"""Gradients on the GPU against FP64 references: the sampling adjoint, the
pose normal equations, Gauss-Newton pose refinement (adjoint vs the plain
FD-Jacobian method) and the vector-Jacobian product of integration."""
import numpy as np
import pytest
import torch

from helpers import oracle_for, small_scene, volume_for

pytestmark = pytest.mark.gpu


def fused_room(w=320, h=240, frames=20, voxel=0.01, trunc=0.1):
    scene = small_scene(w=w, h=h, frames=frames)
    vol = volume_for(scene, voxel=voxel, trunc=trunc, pool_blocks=1 << 17,
                     max_frame_blocks=1 << 17, max_triangles=1 << 22)
    for f in range(frames):
        vol.integrate(*scene.render(f))
    orc = oracle_for(vol, 64)
    e = vol.export_blocks()
    orc.import_blocks(e["xyz"], e["sdf"], e["weight"], e["rgb"])
    return scene, vol, orc, e


@pytest.fixture(scope="module")
def room(gpu):
    return fused_room()


def interior_points(e, voxel, n, seed=0):
    """World points strictly inside voxel cells of observed blocks."""
    rng = np.random.default_rng(seed)
    blocks = e["xyz"][rng.integers(0, len(e["xyz"]), n)]
    local = rng.integers(0, 8, (n, 3))
    frac = rng.uniform(0.05, 0.95, (n, 3))
    q = blocks * 8 + local + frac
    return (q * voxel).astype(np.float32)


def test_sampling_matches_fp64(room):
    scene, vol, orc, e = room
    pts = interior_points(e, vol.params.voxel_size, 20000)
    phi, grad, valid = vol.sdf_sample(pts)
    ophi, ograd, ovalid = orc.sample(pts.astype(np.float64))
    assert valid.sum() > 5000
    assert np.array_equal(valid, ovalid)
    # fp32 world coordinates ~200 voxels from the origin quantise the in-cell
    # position at ~1.5e-5 voxel; |grad| <= ~1 per voxel bounds the sdf error
    assert np.max(np.abs(phi[valid] - ophi[valid])) < 5e-5
    scale = np.abs(ograd[valid]).max()
    assert np.max(np.abs(grad[valid] - ograd[valid])) < 1e-4 * scale


def test_gradient_against_fp64_finite_differences(room):
    scene, vol, orc, e = room
    voxel = vol.params.voxel_size
    pts = interior_points(e, voxel, 3000, seed=1)
    phi, grad, valid = vol.sdf_sample(pts)
    p = pts[valid].astype(np.float64)
    h = 1e-4 * voxel  # stays inside the cell: points are >= 0.05 voxel from faces
    fd = np.zeros_like(p)
    for a in range(3):
        dp = np.zeros(3)
        dp[a] = h
        fp, _, vp = orc.sample(p + dp)
        fm, _, vm = orc.sample(p - dp)
        assert vp.all() and vm.all()
        fd[:, a] = (fp - fm) / (2 * h)
    scale = np.abs(fd).max()
    assert np.max(np.abs(grad[valid] - fd)) < 1e-4 * scale


def test_autograd_binding(room):
    from sdf_autograd import sdf_sample
    scene, vol, orc, e = room
    pts = torch.from_numpy(interior_points(e, vol.params.voxel_size, 4000, seed=2)).cuda()
    pts.requires_grad_(True)
    phi, valid = sdf_sample(pts, vol)
    loss = (phi[valid] ** 2).sum()
    loss.backward()
    p = pts.detach().cpu().numpy().astype(np.float64)
    ophi, ograd, ovalid = orc.sample(p)
    want = np.where(ovalid[:, None], 2 * ophi[:, None] * ograd, 0.0)
    got = pts.grad.cpu().numpy()
    assert np.max(np.abs(got - want)) < 1e-4 * np.abs(want).max()


def test_normal_equations_match_fp64(room):
    scene, vol, orc, e = room
    d, c, p = scene.render(7)
    t = vol.pose_normal_equations(d, p, stride=2)
    o = orc.pose_terms(d, p, stride=2)
    assert abs(t[28] - o[28]) <= 1e-3 * o[28] + 5  # samples at |sdf| == 1 may differ
    assert np.allclose(t[:27], o[:27], rtol=2e-3, atol=2e-3 * np.abs(o[:21]).max())
    fd = vol.pose_normal_equations(d, p, stride=2, method="fd")
    # forward central differences approximate the same Jacobian
    assert np.allclose(fd[:21], t[:21], rtol=0.05, atol=0.05 * np.abs(t[:21]).max())


def perturb(pose, deg, metres, seed):
    """Rotates the camera by `deg` about a random axis through its centre and
    moves the centre by `metres` along a random direction."""
    rng = np.random.default_rng(seed)
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    th = np.deg2rad(deg)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
    dirn = rng.normal(size=3)
    dirn /= np.linalg.norm(dirn)
    out = pose.astype(np.float64).copy()
    out[:3, :3] = R @ out[:3, :3]
    out[:3, 3] = out[:3, 3] + metres * dirn
    return out.astype(np.float32)


def se3_left_exp(xi, P):
    """exp(xi) @ P in FP64 for xi = (v, w)."""
    v, w = np.asarray(xi[:3], np.float64), np.asarray(xi[3:], np.float64)
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        A, B, Cc = 1.0, 0.5, 1.0 / 6.0
    else:
        A, B, Cc = np.sin(th) / th, (1 - np.cos(th)) / th**2, (th - np.sin(th)) / th**3
    R = np.eye(3) + A * K + B * K @ K
    V = np.eye(3) + B * K + Cc * K @ K
    out = np.eye(4)
    out[:3, :3] = R @ P[:3, :3]
    out[:3, 3] = R @ P[:3, 3] + V @ v
    return out


def gn_step(terms, damp=1e-6):
    H = np.zeros((6, 6))
    iu = np.triu_indices(6)
    H[iu] = terms[:21]
    H = H + np.triu(H, 1).T
    H[np.diag_indices(6)] *= 1 + damp
    return -np.linalg.solve(H, terms[21:27])


def pose_error(a, b):
    dt = np.linalg.norm(a[:3, 3].astype(np.float64) - b[:3, 3])
    dR = a[:3, :3].astype(np.float64) @ b[:3, :3].T.astype(np.float64)
    ang = np.degrees(np.arccos(np.clip((np.trace(dR) - 1) / 2, -1, 1)))
    return dt, ang


@pytest.mark.parametrize("method", ["adjoint", "fd"])
def test_pose_refinement_converges(room, method):
    scene, vol, orc, e = room
    for f, seed in ((5, 11), (13, 12)):
        d, c, gt = scene.render(f)
        init = perturb(gt, 2.0, 0.02, seed)
        out, st = vol.pose_refine(d, init, iterations=20, stride=2, method=method)
        dt, ang = pose_error(out, gt)
        assert dt < 2e-3 and ang < 0.1, (method, f, dt, ang, st)
        assert st["final_rmse"] < st["initial_rmse"]


@pytest.mark.parametrize("method", ["adjoint", "fd"])
def test_device_step_matches_host_solve(room, method):
    """One device step (reduce, FP64 Cholesky, exp) equals the host solve of
    the normal equations at the same pose."""
    scene, vol, orc, e = room
    d, c, gt = scene.render(9)
    init = perturb(gt, 1.0, 0.01, 21)
    terms = vol.pose_normal_equations(d, init, stride=2, method=method)
    want = se3_left_exp(gn_step(terms), init.astype(np.float64))
    got, st = vol.pose_refine(d, init, iterations=1, stride=2, method=method)
    assert st["iterations"] == 1 and abs(st["valid_pixels"] - terms[28]) <= 2
    assert np.allclose(got, want, atol=2e-6), np.abs(got - want).max()
    # determinism: the same call gives the same bits
    again, _ = vol.pose_refine(d, init, iterations=1, stride=2, method=method)
    assert np.array_equal(got, again)


def test_refine_stops_without_residuals(room):
    scene, vol, orc, e = room
    d, c, gt = scene.render(3)
    init = perturb(gt, 1.0, 0.01, 5)
    ref, _ = vol.pose_refine(d, init, iterations=20, stride=2)
    empty = np.zeros_like(d)
    out, st = vol.pose_refine(empty, gt, iterations=5, stride=1)
    assert st["iterations"] == 0 and st["valid_pixels"] == 0
    assert np.array_equal(out, gt)
    # the next call on the same handle starts afresh
    again, st = vol.pose_refine(d, init, iterations=20, stride=2)
    assert st["iterations"] == 20 and np.array_equal(again, ref)


@pytest.fixture(scope="module")
def plane_vjp(gpu):
    """Plane scene (constant depth), so pixel re-assignment under a pose
    perturbation cannot change any sample: the engine's VJP of the second
    integration and FP64 finite differences of the oracle's update along a
    random depth direction and a random se(3) direction."""
    from vhsdf import Volume
    from oracle.oracle import Oracle
    W, H, f = 64, 48, 50.0
    params = dict(width=W, height=H, fx=f, fy=f, cx=31.5, cy=23.5, min_depth=0.1, max_depth=4.0,
                  voxel_size=0.01, trunc=0.04, table_log2=16, pool_blocks=1 << 14,
                  max_frame_blocks=1 << 14, max_triangles=1 << 18)
    vol = Volume(**params)
    rgb = np.full((H, W, 3), 100, np.uint8)
    pose0 = np.eye(4, dtype=np.float32)
    vol.integrate(np.full((H, W), 1.0, np.float32), rgb, pose0)
    pre = vol.export_blocks()
    pose1 = perturb(pose0, 1.0, 0.005, 3)
    d1 = np.full((H, W), 1.013, np.float32)
    vol.integrate(d1, rgb, pose1)
    lst = vol.block_list()
    rng = np.random.default_rng(5)
    G = rng.normal(size=(len(lst), 512)).astype(np.float32)
    # The update has jumps where d - z crosses -T (voxel skipped) or +T (dist
    # clamped); finite differences across them measure the jump, not the
    # derivative.  Voxels within 3 mm of either boundary get no upstream
    # gradient, so the loss is smooth over the perturbations below (the
    # pose step moves a voxel by at most 2.4 mm).
    li = np.arange(512)
    vox = (lst[:, None, :] * 8 + np.stack([li & 7, (li >> 3) & 7, li >> 6], -1)[None]) * 0.01
    R, t = pose1[:3, :3].astype(np.float64), pose1[:3, 3].astype(np.float64)
    cam = (vox.reshape(-1, 3) - t) @ R
    zc = cam[:, 2]
    diff = (1.013 - zc).reshape(len(lst), 512)
    G[(np.abs(diff + 0.04) < 3e-3) | (np.abs(diff - 0.04) < 3e-3)] = 0.0
    # voxels whose projection sits on the image border switch in and out too
    # (the pose step moves a projection by at most 0.21 px)
    u = (f * cam[:, 0] / zc + 31.5).reshape(len(lst), 512)
    v = (f * cam[:, 1] / zc + 23.5).reshape(len(lst), 512)
    near = lambda a, b: np.abs(a - b) < 0.25
    G[near(u, -0.5) | near(u, W - 0.5) | near(v, -0.5) | near(v, H - 0.5)] = 0.0
    gd, gp = vol.integrate_vjp(d1, pose1, G)

    key = {tuple(k): i for i, k in enumerate(lst.tolist())}

    def loss(depth, pose):
        o = Oracle(W, H, f, f, 31.5, 23.5, 0.1, 4.0, 0.01, 0.04, precision=64)
        o.import_blocks(pre["xyz"], pre["sdf"], pre["weight"], pre["rgb"])
        o.integrate(depth, rgb, pose)
        ex = o.export(fp64=True)
        total = 0.0
        for i, k in enumerate(ex["xyz"].tolist()):
            j = key.get(tuple(k))
            if j is not None:
                total += float(np.dot(G[j].astype(np.float64), ex["sdf64"][i]))
        return total

    # depth: directional derivative along a random per-pixel direction
    delta = rng.normal(size=(H, W)).astype(np.float32)
    h = 2e-4
    dp, dm = d1 + h * delta, d1 - h * delta
    fd = (loss(dp, pose1) - loss(dm, pose1)) / (2 * h)
    # the float32 images carry the step rounded to float32 (~3e-4 of h per
    # pixel, ~0.5 on this loss): compare against the step actually taken
    step = (dp.astype(np.float64) - dm.astype(np.float64)) / (2 * h)
    # pose: directional derivative along a random se(3) direction.  The
    # oracle takes camera z in fp32 (its decisions are the reference's fp32
    # operations), so every voxel's sdf carries a rounding of ~6e-8 m / T
    # that the difference quotient divides by 2h: summed over the volume's
    # voxels that is ~1 on this loss at h = 2e-4 and ~0.15 at the pose step
    # used here, well inside the tolerance.
    hp = 1.5e-3
    xi = rng.normal(size=6)
    xi /= np.linalg.norm(xi)

    def moved(sign):
        out = pose1.astype(np.float64).copy()
        w, v = sign * hp * xi[3:], sign * hp * xi[:3]
        th = np.linalg.norm(w)
        K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]]) / max(th, 1e-30)
        R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
        out[:3, :3] = R @ out[:3, :3]
        out[:3, 3] = R @ out[:3, 3] + v
        return out.astype(np.float32)

    fdp = (loss(d1, moved(1)) - loss(d1, moved(-1))) / (2 * hp)
    return dict(vol=vol, pre=pre, d1=d1, pose1=pose1, rgb=rgb, G=G, lst=lst, gd=gd, gp=gp,
                fd=fd, step=step, fdp=fdp, xi=xi)


def check_against_fd(c, gd, gp):
    an = float(np.sum(np.asarray(gd, np.float64) * c["step"]))
    assert abs(c["fd"] - an) < 2e-3 * max(1.0, abs(c["fd"])), (c["fd"], an)
    anp = float(np.dot(np.asarray(gp, np.float64), c["xi"]))
    assert abs(c["fdp"] - anp) < 2e-2 * max(1.0, abs(c["fdp"])), (c["fdp"], anp)


def test_integration_vjp_against_fp64_finite_differences(plane_vjp):
    check_against_fd(plane_vjp, plane_vjp["gd"], plane_vjp["gp"])


def test_integration_autograd_binding(plane_vjp):
    """The test-only torch.autograd.Function over the integration update:
    its backward (vh_integrate_vjp) gives the engine's VJP (up to the order
    of its float atomic sums) and matches the FP64 finite differences."""
    from sdf_autograd import integrate_frame
    c = plane_vjp
    depth = torch.tensor(c["d1"], dtype=torch.float32, device="cuda", requires_grad=True)
    delta = torch.zeros(6, dtype=torch.float64, device="cuda", requires_grad=True)
    out = integrate_frame(depth, delta, c["vol"], c["pose1"], c["rgb"], c["pre"])
    assert out.shape == c["G"].shape
    G = c["G"][np.lexsort(c["lst"].T[::-1])]  # the binding's block order
    (out * torch.from_numpy(G).cuda()).sum().backward()
    gd = depth.grad.cpu().numpy()
    gp = delta.grad.cpu().numpy()
    # the VJP sums pixel gradients with float atomics: equal up to summation order
    assert np.allclose(gd, c["gd"], rtol=1e-5, atol=1e-3)
    assert np.allclose(gp, c["gp"], rtol=1e-4, atol=1e-2)
    check_against_fd(c, gd, gp)


def test_batched_refinement(room):
    """vh_pose_refine_batch: one pose equals vh_pose_refine bit for bit; four
    keyframes refined in one launch per step land on their single-pose
    results (the partial sums split over other CTAs, so float-close, not
    bit-equal), repeat to the bit, and agree for host and device depths."""
    import torch
    scene, vol, orc, e = room
    frames = [scene.render(f) for f in (3, 6, 10, 14)]
    inits = [perturb(gt, 2.0, 0.02, 40 + i) for i, (_, _, gt) in enumerate(frames)]
    d0 = frames[0][0]
    one, st1 = vol.pose_refine_batch([d0], [inits[0]], iterations=20, stride=2)
    ref, st_ref = vol.pose_refine(d0, inits[0], iterations=20, stride=2, method="adjoint")
    assert np.array_equal(one[0], ref)
    assert st1[0]["iterations"] == st_ref["iterations"]
    assert st1[0]["final_rmse"] == st_ref["final_rmse"]
    depths = [d for d, _, _ in frames]
    got, st = vol.pose_refine_batch(depths, inits, iterations=20, stride=2)
    again, _ = vol.pose_refine_batch(depths, inits, iterations=20, stride=2)
    assert np.array_equal(got, again)
    u16 = depths[0].dtype == np.uint16  # int16 tensors carry the uint16 bytes
    dev = [torch.from_numpy(d.view(np.int16) if u16 else d).cuda() for d in depths]
    got_d, _ = vol.pose_refine_batch(dev, inits, iterations=20, stride=2,
                                     depth_format="u16" if u16 else None)
    assert np.array_equal(got, got_d)
    for i, (d, _, gt) in enumerate(frames):
        single, _ = vol.pose_refine(d, inits[i], iterations=20, stride=2, method="adjoint")
        dt = np.linalg.norm(got[i][:3, 3].astype(np.float64) - single[:3, 3])
        # small rotation differences from the skew part (arccos of the trace
        # has a ~0.02 deg floor for float32 matrices)
        dR = got[i][:3, :3].astype(np.float64) @ single[:3, :3].T.astype(np.float64)
        w = 0.5 * np.array([dR[2, 1] - dR[1, 2], dR[0, 2] - dR[2, 0], dR[1, 0] - dR[0, 1]])
        ang = np.degrees(np.arcsin(min(1.0, np.linalg.norm(w))))
        assert dt < 1e-4 and ang < 5e-3, (i, dt, ang)
        assert st[i]["final_rmse"] < st[i]["initial_rmse"]
