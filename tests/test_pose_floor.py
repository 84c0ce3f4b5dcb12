"""Where Gauss-Newton pose refinement on a fused TSDF ends when it starts AT
the ground-truth pose (the floor that bounds refinement accuracy), measured
with the FP64 oracle on noise-free depth of the 4x4x3 m room with 3 spheres
(320x240, 24 frames, truncation 0.1 m): it is a fraction of a voxel and
shrinks in proportion to the voxel size (about 0.16 voxel: 3.2, 1.7 and
0.75 mm at 20, 10 and 5 mm voxels).  So the floor comes from the
voxel-scale discretisation of projective fusion, not from depth noise, and
the refinement benchmark's 1 mm / 0.05 deg target at 5 mm voxels sits
at about this floor."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from vhsdf import synth


def se3_exp(xi):
    v, w = xi[:3], xi[3:]
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        R, V = np.eye(3) + K, np.eye(3) + 0.5 * K
    else:
        R = np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K
        V = np.eye(3) + (1 - np.cos(th)) / th ** 2 * K + (th - np.sin(th)) / th ** 3 * K @ K
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, V @ v
    return T


def refine(orc, depth, pose, iterations=20):
    """Gauss-Newton on the oracle's FP64 normal equations, left perturbation
    (the engine's vh_pose_refine, restated in numpy)."""
    P = np.asarray(pose, np.float64).copy()
    for _ in range(iterations):
        t = orc.pose_terms(depth, P)
        if t[28] < 6:
            break
        A = np.zeros((6, 6))
        iu = np.triu_indices(6)
        A[iu] = t[:21]
        A = A + A.T - np.diag(np.diag(A))
        P = se3_exp(-np.linalg.solve(A, t[21:27])) @ P
    return P


def pose_error_mm(P, G):
    return 1000.0 * np.linalg.norm(P[:3, 3] - np.asarray(G, np.float64)[:3, 3])


@pytest.fixture(scope="module")
def floors():
    w, h, nf = 320, 240, 24
    s = synth.Scene(kind=1, seed=0, num_frames=nf, width=w, height=h)
    frames = [s.render(f, noise=False) for f in range(nf)]
    out = {}
    for vox in (0.02, 0.01, 0.005):
        orc = Oracle(w, h, s.fx, s.fy, s.cx, s.cy, min_depth=0.1, max_depth=4.5, voxel_size=vox,
                     trunc=0.1, precision=64)
        for d, c, p in frames:
            orc.integrate(d, c, p)
        errs = [pose_error_mm(refine(orc, frames[f][0], frames[f][2]), frames[f][2])
                for f in range(0, nf, 3)]
        out[vox] = float(np.median(errs))
    return out


def test_floor_is_a_fraction_of_a_voxel(floors):
    for vox, e in floors.items():
        assert 0.08 <= e / (1000 * vox) <= 0.25, (vox, e)


def test_floor_shrinks_with_the_voxel(floors):
    assert 0.35 <= floors[0.01] / floors[0.02] <= 0.7, floors
    assert 0.35 <= floors[0.005] / floors[0.01] <= 0.7, floors
