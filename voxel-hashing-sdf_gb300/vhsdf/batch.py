"""Many independent scenes stepped together over the C ABI (vh_batch_*).

Every scene keeps its own parameters (image size, intrinsics, voxel size,
truncation, table and pool sizes).  One batched step runs allocation,
integration and optionally the frame's marching cubes for every scene that
has a frame, each stage as one launch over all those scenes.  Nothing here
computes anything itself.
"""
import ctypes as C

import numpy as np

from . import _native as N
from .engine import Volume, _depth_arg, _rgb_arg


class _Scene(Volume):
    """A scene of a batch: a Volume whose handle the batch owns."""

    def __init__(self, batch, index, params):
        self._L = N.lib()
        self.params = params
        self._batch = batch  # keeps the batch (and the handle) alive
        self._h = C.c_void_p(self._L.vh_batch_scene(batch._b, index))

    def close(self):
        self._h = None


class Batch:
    def __init__(self, scenes):
        """scenes: one dict of vh_params fields per scene.  VH_FLAG_BATCH_FUSED
        in the first scene's flags runs each step as one persistent launch
        over every stage of every scene (the same results as the staged
        launches)."""
        self._L = N.lib()
        n = len(scenes)
        arr = (N.VhParams * n)()
        for i, prm in enumerate(scenes):
            self._L.vh_params_default(C.byref(arr[i]))
            for k, v in prm.items():
                if not hasattr(arr[i], k):
                    raise TypeError(f"unknown parameter {k}")
                setattr(arr[i], k, v)
        b = C.c_void_p()
        N.check(self._L.vh_batch_create(arr, n, C.byref(b)))
        self._b = b
        self.n = n
        self._params = arr
        self._scenes = [_Scene(self, i, arr[i]) for i in range(n)]

    def close(self):
        if getattr(self, "_b", None):
            for s in self._scenes:
                s.close()
            self._L.vh_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return self.n

    def scene(self, i):
        return self._scenes[i]

    def process(self, frames, with_mesh=False, depth_format=None):
        """frames[i]: (depth, rgb, c2w) for scene i, or None (no frame this
        step).  Depths share one format; all arrays host (numpy) or all device
        (CUDA tensors)."""
        if len(frames) != self.n:
            raise ValueError("one entry per scene")
        dptr = (C.c_void_p * self.n)()
        cptr = (C.c_void_p * self.n)()
        poses = np.zeros((self.n, 16), np.float32)
        keep, fmt, mem = [], None, None
        for i, fr in enumerate(frames):
            if fr is None:
                continue
            d, f = _depth_arg(fr[0], self._params[i], depth_format)
            c = _rgb_arg(fr[1], self._params[i])
            if fmt is not None and (f != fmt or d.mem != mem):
                raise ValueError("all frames of a step share depth format and memory kind")
            if d.mem != c.mem:
                raise ValueError("depth and rgb must both be host or both be device arrays")
            fmt, mem = f, d.mem
            keep += [d, c]
            dptr[i], cptr[i] = d.ptr, c.ptr
            poses[i] = np.asarray(fr[2], np.float32).reshape(16)
        if fmt is None:
            return
        N.check(self._L.vh_batch_process(self._b, dptr, fmt, cptr, poses.ctypes.data, mem,
                                         int(bool(with_mesh))))

    def sync(self):
        """(per-scene status codes, per-scene stats dicts) after the last step."""
        st = (C.c_int32 * self.n)()
        stats = (N.VhStats * self.n)()
        self._L.vh_batch_sync(self._b, st, stats)
        names = [f for f, _ in N.VhStats._fields_]
        return list(st), [{f: getattr(s, f) for f in names} for s in stats]
