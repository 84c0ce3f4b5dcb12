"""CPU oracle of the TSDF path - TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always as the checker.  It wraps
oracle/vh_oracle.cpp (a plain C++ restatement of the reference's camera math,
integration rule and marching cubes, cited line by line there) and feeds it
the marching-cubes tables pinned in tests/golden/ref_golden.json, which were
produced by the reference's own code.
"""
import ctypes as C
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "lib", "libvh_oracle.so")
GOLDEN = os.path.join(REPO, "tests", "golden", "ref_golden.json")

_lib = None
_tables = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"oracle library missing: {LIB_PATH}")
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.vho_create.restype = P
        L.vho_create.argtypes = [P, P, P, P, P, C.c_int32]
        L.vho_destroy.argtypes = [P]
        L.vho_set_threads.argtypes = [C.c_int32]
        L.vho_max_threads.restype = C.c_int32
        L.vho_integrate.restype = C.c_int64
        L.vho_integrate.argtypes = [P, P, P, P]
        L.vho_band_blocks.restype = C.c_int64
        L.vho_band_blocks.argtypes = [P, P, P, P, P, C.c_int64]
        L.vho_num_blocks.restype = C.c_int64
        L.vho_num_blocks.argtypes = [P]
        L.vho_frame_blocks.restype = C.c_int64
        L.vho_frame_blocks.argtypes = [P]
        L.vho_last_counts.argtypes = [P, P]
        L.vho_export.restype = C.c_int64
        L.vho_export.argtypes = [P, C.c_int32, P, P, P, P, P, P]
        L.vho_import.argtypes = [P, P, P, P, P, C.c_int64]
        L.vho_set_frame.argtypes = [P, P, C.c_int64]
        L.vho_mc.restype = C.c_int64
        L.vho_mc.argtypes = [P, C.c_int32]
        L.vho_mc_copy.restype = C.c_int64
        L.vho_mc_copy.argtypes = [P, P, P, P, P, C.c_int64]
        L.vho_sample.argtypes = [P, P, C.c_int64, C.c_double, P, P, P]
        L.vho_pose_terms.argtypes = [P, P, P, C.c_int32, C.c_double, P]
        L.vho_raycast.argtypes = [P, P, C.c_double, P, P]
        _lib = L
    return _lib


def tables():
    """MC tables as produced by the reference (idxMap, edgeTable, triTable)."""
    global _tables
    if _tables is None:
        with open(GOLDEN) as f:
            d = json.load(f)
        _tables = (np.array(d["idx_map"], np.int32), np.array(d["edge_table"], np.int32),
                   np.array(d["tri_table"], np.int32))
    return _tables


def depth_to_metres(depth, depth_scale=0.001):
    """uint16 depth -> float32 metres with one fp32 multiply (as the engine)."""
    if depth.dtype == np.uint16:
        return depth.astype(np.float32) * np.float32(depth_scale)
    return np.ascontiguousarray(depth, np.float32)


class Oracle:
    """One CPU volume. precision 32: bit-exact fp32 accumulation; 64: FP64."""

    def __init__(self, width, height, fx, fy, cx, cy, min_depth=0.1, max_depth=10.0,
                 voxel_size=0.036, trunc=0.18, mc_min_weight=1.0, depth_scale=0.001,
                 precision=64):
        self._L = lib()
        self.depth_scale = depth_scale
        self.fp = np.array([fx, fy, cx, cy, min_depth, max_depth, voxel_size, trunc,
                            mc_min_weight], np.float32)
        self.ip = np.array([width, height], np.int32)
        idx, edge, tri = tables()
        self._h = self._L.vho_create(self.fp.ctypes.data, self.ip.ctypes.data, idx.ctypes.data,
                                     edge.ctypes.data, tri.ctypes.data, precision)
        self.precision = precision

    @classmethod
    def from_volume_params(cls, p, precision=64):
        return cls(p.width, p.height, p.fx, p.fy, p.cx, p.cy, p.min_depth, p.max_depth,
                   p.voxel_size, p.trunc, p.mc_min_weight, p.depth_scale, precision)

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.vho_destroy(self._h)
            self._h = None

    @staticmethod
    def set_threads(n):
        lib().vho_set_threads(int(n))

    @staticmethod
    def max_threads():
        return lib().vho_max_threads()

    def integrate(self, depth, rgb, c2w):
        d = depth_to_metres(depth, self.depth_scale)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        pose = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(16))
        return self._L.vho_integrate(self._h, d.ctypes.data, rgb.ctypes.data, pose.ctypes.data)

    def band_blocks(self, depth, c2w):
        d = depth_to_metres(depth, self.depth_scale)
        pose = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(16))
        n = self._L.vho_band_blocks(self.fp.ctypes.data, self.ip.ctypes.data, d.ctypes.data,
                                    pose.ctypes.data, None, 0)
        out = np.empty((n, 3), np.int32)
        self._L.vho_band_blocks(self.fp.ctypes.data, self.ip.ctypes.data, d.ctypes.data,
                                pose.ctypes.data, out.ctypes.data, n)
        return out

    def counts(self):
        out = np.zeros(3, np.int64)
        self._L.vho_last_counts(self._h, out.ctypes.data)
        return {"new_blocks": int(out[0]), "voxels_updated": int(out[1]),
                "range_errors": int(out[2])}

    def num_blocks(self):
        return self._L.vho_num_blocks(self._h)

    def export(self, frame=False, fp64=False):
        """Blocks sorted by packed key (x, y, z order of the key bits)."""
        n = self._L.vho_frame_blocks(self._h) if frame else self._L.vho_num_blocks(self._h)
        xyz = np.empty((n, 3), np.int32)
        sdf = np.empty((n, 512), np.float32)
        w = np.empty((n, 512), np.float32)
        rgb = np.empty((n, 512, 3), np.uint8)
        sdf64 = np.empty((n, 512), np.float64) if fp64 else None
        w64 = np.empty((n, 512), np.float64) if fp64 else None
        self._L.vho_export(self._h, int(frame), xyz.ctypes.data, sdf.ctypes.data, w.ctypes.data,
                           rgb.ctypes.data, sdf64.ctypes.data if fp64 else None,
                           w64.ctypes.data if fp64 else None)
        out = {"xyz": xyz, "sdf": sdf, "weight": w, "rgb": rgb}
        if fp64:
            out["sdf64"] = sdf64
            out["weight64"] = w64
        return out

    def import_blocks(self, xyz, sdf, weight, rgb):
        xyz = np.ascontiguousarray(xyz, np.int32)
        sdf = np.ascontiguousarray(sdf, np.float32)
        weight = np.ascontiguousarray(weight, np.float32)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        self._L.vho_import(self._h, xyz.ctypes.data, sdf.ctypes.data, weight.ctypes.data,
                           rgb.ctypes.data, xyz.shape[0])

    def set_frame(self, xyz):
        xyz = np.ascontiguousarray(xyz, np.int32)
        self._L.vho_set_frame(self._h, xyz.ctypes.data, xyz.shape[0])

    def marching_cubes(self, scope="all"):
        n = self._L.vho_mc(self._h, int(scope == "all"))
        xyz = np.empty((n, 3, 3), np.float32)
        rgb = np.empty((n, 3, 3), np.uint8)
        xyz64 = np.empty((n, 3, 3), np.float64)
        cube = np.empty((n, 4), np.int32)
        self._L.vho_mc_copy(self._h, xyz.ctypes.data, rgb.ctypes.data, xyz64.ctypes.data,
                            cube.ctypes.data, n)
        return {"xyz": xyz, "rgb": rgb, "xyz64": xyz64, "cube": cube}

    def sample(self, xyz, min_weight=1.0):
        """FP64 trilinear sdf and gradient at world points (n x 3)."""
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        n = xyz.shape[0]
        phi = np.empty(n, np.float64)
        grad = np.empty((n, 3), np.float64)
        valid = np.empty(n, np.uint8)
        self._L.vho_sample(self._h, xyz.ctypes.data, n, float(min_weight), phi.ctypes.data,
                           grad.ctypes.data, valid.ctypes.data)
        return phi, grad, valid.astype(bool)

    def raycast(self, c2w, min_weight=1.0):
        """FP64 ray cast of the fused surface: (depth [H,W], normals [H,W,3])."""
        P = np.ascontiguousarray(np.asarray(c2w, np.float64).reshape(4, 4)[:3].reshape(12))
        h, w = int(self.ip[1]), int(self.ip[0])
        depth = np.empty((h, w), np.float64)
        normal = np.empty((h, w, 3), np.float64)
        self._L.vho_raycast(self._h, P.ctypes.data, float(min_weight), depth.ctypes.data,
                            normal.ctypes.data)
        return depth, normal

    def pose_terms(self, depth, c2w, stride=1, min_weight=1.0):
        """FP64 Gauss-Newton terms of the SDF residuals of a depth image."""
        d = depth_to_metres(depth, self.depth_scale)
        P = np.ascontiguousarray(np.asarray(c2w, np.float64).reshape(4, 4)[:3].reshape(12))
        out = np.empty(29, np.float64)
        self._L.vho_pose_terms(self._h, d.ctypes.data, P.ctypes.data, int(stride),
                               float(min_weight), out.ctypes.data)
        return out
