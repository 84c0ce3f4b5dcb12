"""Known-answer tests of the CPU oracle (no GPU)."""
import numpy as np
import pytest

from oracle.oracle import Oracle

W, H = 64, 48
FX = FY = 50.0
CX, CY = 31.5, 23.5
V, T = 0.01, 0.04


def plane_frame(d):
    depth = np.full((H, W), d, np.float32)
    rgb = np.zeros((H, W, 3), np.uint8)
    rgb[..., 0] = 200
    rgb[..., 1] = np.arange(W, dtype=np.uint8)[None, :]
    rgb[..., 2] = 7
    return depth, rgb, np.eye(4, dtype=np.float32)


def grid_of(z):
    return np.floor(((np.float32(z) / np.float32(V)) + np.float32(0.5)) * np.float32(0.125))


@pytest.mark.parametrize("precision", [32, 64])
def test_fronto_parallel_plane_sdf(precision):
    d = 1.2345
    o = Oracle(W, H, FX, FY, CX, CY, min_depth=0.1, max_depth=4.0, voxel_size=V, trunc=T,
               precision=precision)
    depth, rgb, pose = plane_frame(d)
    o.integrate(depth, rgb, pose)
    e = o.export()
    assert len(e["xyz"]) > 0
    # every allocated block lies in the band's z-range of blocks
    bz = set(e["xyz"][:, 2].tolist())
    lo, hi = grid_of(np.float32(d) - np.float32(T)), grid_of(np.float32(d) + np.float32(T))
    assert bz == set(range(int(lo), int(hi) + 1))
    li = np.arange(512)
    xs, ys, zs = li & 7, (li >> 3) & 7, li >> 6
    iz = e["xyz"][:, 2:3] * 8 + zs[None, :]
    ix = e["xyz"][:, 0:1] * 8 + xs[None, :]
    iy = e["xyz"][:, 1:2] * 8 + ys[None, :]
    z = iz.astype(np.float64) * V
    u = FX * (ix * V) / z + CX
    v = FY * (iy * V) / z + CY
    inside = (u > 0.6) & (u < W - 1.6) & (v > 0.6) & (v < H - 1.6)
    diff = np.float64(np.float32(d)) - z
    upd = inside & (diff > -T + 1e-4)
    skip = inside & (diff <= -T - 1e-4)
    assert upd.sum() > 1000
    expect = np.minimum(1.0, diff / T)
    assert np.all(e["weight"][upd] == 1.0)
    assert np.all(e["weight"][skip] == 0.0)
    # z carries fp32 rounding of the camera transform (~1e-7 m at 1.2 m);
    # dividing by T = 0.04 m scales that to a few 1e-6 in sdf units.
    assert np.max(np.abs(e["sdf"][upd] - expect[upd])) < 5e-6
    # colour of the single observation is the pixel's colour
    assert np.all(e["rgb"][upd][:, 0] == 200) and np.all(e["rgb"][upd][:, 2] == 7)


def test_running_average_repeats():
    o = Oracle(W, H, FX, FY, CX, CY, max_depth=4.0, voxel_size=V, trunc=T, precision=64)
    depth, rgb, pose = plane_frame(0.9)
    o.integrate(depth, rgb, pose)
    first = o.export()
    for _ in range(2):
        o.integrate(depth, rgb, pose)
    e = o.export()
    m = first["weight"] > 0
    assert np.all(e["weight"][m] == 3.0)
    assert np.max(np.abs(e["sdf"][m] - first["sdf"][m])) < 1e-6
    assert np.array_equal(e["rgb"], first["rgb"])


def test_weighted_average_two_depths():
    o = Oracle(W, H, FX, FY, CX, CY, max_depth=4.0, voxel_size=V, trunc=T, precision=64)
    d1, rgb, pose = plane_frame(1.0)
    d2 = np.full_like(d1, 1.02)
    o.integrate(d1, rgb, pose)
    o.integrate(d2, rgb, pose)
    e = o.export(fp64=True)
    li = np.arange(512)
    z = (e["xyz"][:, 2:3] * 8 + (li >> 6)[None, :]) * V
    both = e["weight64"] == 2
    s1 = np.minimum(1, (np.float32(1.0) - z) / T)
    s2 = np.minimum(1, (np.float32(1.02) - z) / T)
    ok = both & (z < 0.98 + T - 1e-3)
    assert ok.sum() > 100
    assert np.max(np.abs(e["sdf64"][ok] - 0.5 * (s1 + s2)[ok])) < 1e-5


def test_empty_depth_allocates_nothing():
    o = Oracle(W, H, FX, FY, CX, CY, max_depth=4.0, voxel_size=V, trunc=T)
    depth = np.zeros((H, W), np.float32)
    rgb = np.zeros((H, W, 3), np.uint8)
    assert o.integrate(depth, rgb, np.eye(4, dtype=np.float32)) == 0
    assert o.num_blocks() == 0
    assert len(o.marching_cubes()["xyz"]) == 0


def test_mc_vertices_stay_in_their_cube_and_fp64_agrees():
    from vhsdf import synth
    s = synth.Scene(kind=1, seed=0, num_frames=20, width=160, height=120)
    o32 = Oracle(160, 120, s.fx, s.fy, s.cx, s.cy, max_depth=4.5, voxel_size=0.02, trunc=0.08,
                 precision=32)
    o64 = Oracle(160, 120, s.fx, s.fy, s.cx, s.cy, max_depth=4.5, voxel_size=0.02, trunc=0.08,
                 precision=64)
    for f in range(3):
        d, c, p = s.render(f)
        o32.integrate(d, c, p)
        o64.integrate(d, c, p)
    a, b = o32.export(), o64.export(fp64=True)
    assert np.array_equal(a["xyz"], b["xyz"])
    assert np.array_equal(a["weight"], b["weight"])
    assert np.max(np.abs(a["sdf"].astype(np.float64) - b["sdf64"])) < 1e-5
    assert np.max(np.abs(a["rgb"].astype(int) - b["rgb"].astype(int))) <= 1
    m = o64.marching_cubes("all")
    n = len(m["xyz"])
    assert n > 1000
    lo = m["cube"][:, None, :3].astype(np.float32)
    assert np.all(m["xyz"] >= lo - 1e-4) and np.all(m["xyz"] <= lo + 1 + 1e-4)
    assert np.max(np.abs(m["xyz"] - m["xyz64"])) < 1e-3


@pytest.mark.parametrize("precision", [32, 64])
def test_raycast_of_a_plane_returns_its_depth(precision):
    """The truncated SDF of a fronto-parallel plane is linear in z inside the
    band, so trilinear sampling and the march's linear crossing are exact:
    the cast depth is the plane's depth and the normal faces the camera."""
    d = 1.2345
    o = Oracle(W, H, FX, FY, CX, CY, min_depth=0.1, max_depth=4.0, voxel_size=V, trunc=T,
               precision=precision)
    depth, rgb, pose = plane_frame(d)
    o.integrate(depth, rgb, pose)
    cast, normal = o.raycast(pose)
    inner = (slice(8, H - 8), slice(8, W - 8))
    assert np.all(cast[inner] > 0)
    assert np.max(np.abs(cast[inner] - np.float64(np.float32(d)))) < 1e-5
    assert np.max(np.abs(normal[inner] - np.array([0.0, 0.0, -1.0]))) < 1e-6
    # rays that leave the observed frustum's band before crossing miss
    assert np.all((cast == 0) | (np.abs(cast - d) < 1e-4))


def test_pose_terms_of_a_plane_have_closed_form():
    """A depth image offset by delta from the fused plane: every residual is
    T * phi = -delta, the Jacobian row is (0, 0, -1, -y, x, 0), so the sums
    are count, count * delta and count * delta^2."""
    d, delta = 1.2345, 0.005
    o = Oracle(W, H, FX, FY, CX, CY, min_depth=0.1, max_depth=4.0, voxel_size=V, trunc=T,
               precision=64)
    depth, rgb, pose = plane_frame(d)
    o.integrate(depth, rgb, pose)
    obs = np.full((H, W), np.float32(d + delta), np.float32)
    t = o.pose_terms(obs, pose)
    n = t[28]
    assert n > 0.5 * W * H
    row = {a: 6 * a - a * (a - 1) // 2 for a in range(6)}   # packed upper triangle
    dz = np.float64(np.float32(d + delta)) - np.float64(np.float32(d))
    # the gradient is a difference of fp32-stored sdf values over a voxel
    assert abs(t[row[2]] - n) < 1e-5 * n                    # J_tz . J_tz
    assert abs(t[21 + 2] - n * dz) < 1e-4 * n * dz          # J_tz . r
    assert abs(t[27] - n * dz * dz) < 2e-4 * n * dz * dz     # r . r
    for a in (0, 1):                                         # no in-plane gradient
        assert abs(t[row[a]]) < 1e-9 and abs(t[21 + a]) < 1e-9
    assert abs(t[row[5]]) < 1e-9                             # J_rz vanishes


@pytest.mark.parametrize("c", [7.3, 7.0, 0.5])
def test_mc_of_a_plane_has_closed_form(c):
    """sdf = (c - z) / T over 2x2x2 blocks (voxel units): every cube whose
    eight corners exist (origins 0..14 on each axis) and whose z-span holds
    the crossing emits two triangles, every vertex on z = c (the sdf is
    linear, so the interpolation is exact; a corner exactly on the plane
    is not negative and snaps the vertex onto itself)."""
    o = Oracle(W, H, FX, FY, CX, CY, max_depth=4.0, voxel_size=V, trunc=T, precision=32)
    bx, by, bz = np.meshgrid(range(2), range(2), range(2), indexing="ij")
    xyz = np.stack([bx.ravel(), by.ravel(), bz.ravel()], -1).astype(np.int32)
    li = np.arange(512)
    z = (xyz[:, 2:3] * 8 + (li >> 6)[None, :]).astype(np.float32)
    sdf = ((np.float32(c) - z) * np.float32(0.25)).astype(np.float32)  # T = 4 voxels
    w = np.ones_like(sdf)
    rgb = np.full((len(xyz), 512, 3), 9, np.uint8)
    o.import_blocks(xyz, sdf, w, rgb)
    m = o.marching_cubes("all")
    k = int(np.floor(c))  # the cube layer whose z-span [k, k + 1) holds c
    assert len(m["xyz"]) == 15 * 15 * 2
    assert np.all(m["cube"][:, 2] == k)
    assert np.max(np.abs(m["xyz"][..., 2] - np.float32(c))) < 1e-5
    # the triangles tile the 15 x 15 voxel square exactly once
    e1 = m["xyz64"][:, 1, :2] - m["xyz64"][:, 0, :2]
    e2 = m["xyz64"][:, 2, :2] - m["xyz64"][:, 0, :2]
    area = 0.5 * np.abs(e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
    assert abs(area.sum() - 15.0 * 15.0) < 1e-6
    # one winding: every triangle faces the positive-sdf (observed) side, -z
    n = np.cross(m["xyz64"][:, 1] - m["xyz64"][:, 0], m["xyz64"][:, 2] - m["xyz64"][:, 0])
    assert np.all(n[:, 2] < 0)
    assert np.all(m["rgb"] == 9)


def test_mc_of_a_sphere_is_a_closed_genus_zero_surface():
    """Truncated distance to a sphere (radius 5.2 voxels) over 2x2x2 blocks:
    with vertices merged by position (FP64 vertices) the mesh is a closed
    2-manifold of Euler characteristic 2, every edge in exactly two
    triangles, every vertex within 0.05 voxel of the sphere.  The fp32
    vertices of one edge, interpolated from either end by the two cubes
    that share it, differ by at most one ulp, so the reference's
    exact-equality merge (tsdf2mesh) can split a vertex in two."""
    o = Oracle(W, H, FX, FY, CX, CY, max_depth=4.0, voxel_size=V, trunc=T, precision=32)
    bx, by, bz = np.meshgrid(range(2), range(2), range(2), indexing="ij")
    xyz = np.stack([bx.ravel(), by.ravel(), bz.ravel()], -1).astype(np.int32)
    li = np.arange(512)
    pts = np.stack([xyz[:, None, 0] * 8 + (li & 7)[None], xyz[:, None, 1] * 8 + ((li >> 3) & 7)[None],
                    xyz[:, None, 2] * 8 + (li >> 6)[None]], -1).astype(np.float64)
    centre, r = np.array([8.3, 8.1, 7.9]), 5.2
    sdf = np.clip((np.linalg.norm(pts - centre, axis=-1) - r) / 4.0, -1, 1).astype(np.float32)
    o.import_blocks(xyz, sdf, np.ones_like(sdf), np.full((len(xyz), 512, 3), 9, np.uint8))
    m = o.marching_cubes("all")
    nf = len(m["xyz"])
    assert nf > 500
    key = np.round(m["xyz64"].reshape(-1, 3) * 1e5).astype(np.int64)
    verts, faces = np.unique(key, axis=0, return_inverse=True)
    faces = faces.reshape(-1, 3)
    edges = np.sort(np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]]), axis=1)
    ue, count = np.unique(edges, axis=0, return_counts=True)
    assert np.all(count == 2)
    assert len(verts) - len(ue) + nf == 2
    rad = np.linalg.norm(m["xyz64"].reshape(-1, 3) - centre, axis=1)
    assert np.max(np.abs(rad - r)) < 0.05
    f32 = m["xyz"].reshape(-1, 3)
    ulp = np.spacing(np.abs(f32).max())
    for g in range(len(verts)):
        same = f32[faces.ravel() == g]
        assert np.max(np.abs(same - same[0])) <= ulp


def test_sample_gradient_equals_differences_of_the_sample():
    """Within one trilinear cell the oracle's sdf sample is a polynomial, so
    its reported gradient equals central differences of the sample (points
    and steps chosen so that x +- h stays in the same cell)."""
    from vhsdf import synth
    s = synth.Scene(kind=1, seed=0, num_frames=4, width=160, height=120)
    o = Oracle(160, 120, s.fx, s.fy, s.cx, s.cy, max_depth=4.5, voxel_size=0.02, trunc=0.08,
               precision=64)
    for f in range(3):
        o.integrate(*s.render(f))
    e = o.export()
    rng = np.random.default_rng(3)
    blk = e["xyz"][rng.integers(0, len(e["xyz"]), 400)]
    cell = blk * 8 + rng.integers(0, 7, (400, 3))          # a cell inside the block
    frac = rng.uniform(0.2, 0.8, (400, 3))
    pts = (cell + frac) * 0.02
    phi, grad, valid = o.sample(pts)
    h = 1e-5
    checked = 0
    for a in range(3):
        d = np.zeros(3)
        d[a] = h
        pp, _, vp = o.sample(pts + d)
        pm, _, vm = o.sample(pts - d)
        ok = valid & vp & vm
        fd = (pp - pm) / (2 * h)
        assert np.max(np.abs(fd[ok] - grad[ok, a])) < 1e-6 * max(1.0, np.max(np.abs(grad[ok, a])))
        checked += ok.sum()
    assert checked > 300


def _exp_se3(xi):
    """exp of xi = (v, w): rotation by Rodrigues' formula, translation v."""
    v, w = xi[:3], xi[3:]
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    R = np.eye(3) + K if th < 1e-300 else (np.eye(3) + np.sin(th) / th * K
                                           + (1 - np.cos(th)) / th ** 2 * K @ K)
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, v
    return T


def test_pose_terms_gradient_equals_differences_of_the_cost():
    """For the left perturbation c2w -> exp(xi) c2w the oracle's J^T r is the
    gradient of half the summed squared residuals: central differences of
    that sum along random se(3) directions agree with (J^T r) . xi.  The
    trilinear sample has slope jumps at cell faces; with ~18k residuals a
    step of 1e-6 carries a few of them (errors ~1e-3), a step of 1e-8 none
    here, and its rounding stays far below the tolerance."""
    from vhsdf import synth
    s = synth.Scene(kind=1, seed=0, num_frames=20, width=160, height=120)
    o = Oracle(160, 120, s.fx, s.fy, s.cx, s.cy, max_depth=4.5, voxel_size=0.02, trunc=0.08,
               precision=64)
    for f in range(0, 8):
        o.integrate(*s.render(f))
    d, _, P = s.render(3)
    P0 = _exp_se3(np.array([0.002, -0.001, 0.0015, 0.002, -0.001, 0.0005])) @ P.astype(np.float64)
    t0 = o.pose_terms(d, P0)
    assert t0[28] > 5000 and t0[27] > 0
    rng = np.random.default_rng(1)
    h = 1e-8
    for _ in range(4):
        xi = rng.normal(size=6)
        xi /= np.linalg.norm(xi)
        tp, tm = o.pose_terms(d, _exp_se3(h * xi) @ P0), o.pose_terms(d, _exp_se3(-h * xi) @ P0)
        assert tp[28] == tm[28] == t0[28]  # same residual set on both sides
        fd = (tp[27] - tm[27]) / (4 * h)
        an = float(np.dot(t0[21:27], xi))
        assert abs(fd - an) < 1e-5 * max(1.0, abs(an)), (fd, an)
