"""Seeded synthetic RGB-D streams (stand-in for the ScanNet frames the
reference reads with SaveFrame::frameLoad, src/SaveFrame.cpp:154-218).

Scene kinds are documented in synth/vh_synth.cpp.  Frames come out as the
reference's inputs: uint16 millimetre depth, interleaved RGB bytes and a
row-major camera-to-world matrix.
"""
import numpy as np

from . import _native as N

# fx=fy=525, cx=319.5, cy=239.5 at 640 x 480, scaled for other sizes.
def intrinsics(width=640, height=480):
    s = width / 640.0
    return 525.0 * s, 525.0 * s, (width - 1) / 2.0, (height - 1) / 2.0


class Scene:
    def __init__(self, kind, seed, num_frames, width=640, height=480, fx=None, fy=None,
                 cx=None, cy=None):
        dfx, dfy, dcx, dcy = intrinsics(width, height)
        self.width, self.height = width, height
        self.fx = dfx if fx is None else fx
        self.fy = dfy if fy is None else fy
        self.cx = dcx if cx is None else cx
        self.cy = dcy if cy is None else cy
        self._L = N.synth_lib()
        self._h = self._L.vhs_create(kind, seed, width, height, self.fx, self.fy, self.cx,
                                     self.cy, num_frames)
        if not self._h:
            raise ValueError("invalid scene parameters")
        self.num_frames = self._L.vhs_num_frames(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.vhs_destroy(self._h)
            self._h = None

    @property
    def num_objects(self):
        return self._L.vhs_num_objects(self._h)

    def bounds(self):
        b = np.empty(6, np.float32)
        self._L.vhs_bounds(self._h, b.ctypes.data)
        return b[:3].copy(), b[3:].copy()

    def render(self, f, noise=True):
        depth = np.empty((self.height, self.width), np.uint16)
        rgb = np.empty((self.height, self.width, 3), np.uint8)
        c2w = np.empty((4, 4), np.float32)
        if self._L.vhs_render(self._h, f, depth.ctypes.data, rgb.ctypes.data, c2w.ctypes.data,
                              int(noise)) != 0:
            raise IndexError(f"frame {f} out of range")
        return depth, rgb, c2w


# Workloads named by what they are (sizes from the benchmark definitions).
SMALL_ROOM = dict(kind=1, seed=0, num_frames=20)          # 4x4x3 m room, 3 spheres
LONG_STREAM = dict(kind=2, seed=2, num_frames=500)        # 8x8x3 m room, 40 objects
