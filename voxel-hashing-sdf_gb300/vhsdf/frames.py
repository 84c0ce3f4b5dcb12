"""RGB-D frames stored in the reference's folder layout, read into the
arrays Volume.integrate takes.

The reference's frame store (src/SaveFrame.cpp:44-52, 154-218) keeps frame
`i` of a sequence as

    <root>/RGB/<i>.jpg     colour (its writer stores <i>.png)
    <root>/depth/<i>.png   16-bit grayscale depth in millimetres
    <root>/tcw/<i>.txt     16 numbers: a row-major 4 x 4 camera-to-world pose

and its application loop (src/main.cpp:242-258) fuses frames 0, 20, 40, ...
below 2025, stopping once five of them were missing.  FrameFolder.load
returns one frame through the library's vh_load_frame (which decodes with
vh_decode_depth_png, vh_decode_colour_jpeg / vh_decode_colour_png and
vh_resize_colour, and reads the pose as the reference does, each number
as the nearest float); FrameFolder.frames walks the schedule.

Differences from the reference's loader, by design:
- depth stays uint16 millimetres (VH_DEPTH_U16_MM); the reference converts
  it to float metres on the host (src/SaveFrame.cpp:179-180), the engine
  scales it inside the allocation kernel;
- colour is resized to the depth image's size; the reference resizes it to
  640 x 480 (src/SaveFrame.cpp:171), the depth size of its data;
- the pose is the file's matrix with the last row set to (0, 0, 0, 1), as
  PointCloudGenerator::Reproject sets it (src/PointCloudGenerator.cpp:
  118-125); the reference inverts the matrix on loading and inverts it back
  before fusing (src/SaveFrame.cpp:206, src/PointCloudGenerator.cpp:140),
  which returns the same matrix up to float rounding;
- colour files are decoded by their content, JPEG or PNG, whatever their
  name (the reference's writer stores PNG under <i>.png, its loader reads
  <i>.jpg).
"""
import ctypes as C
import os
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from typing import NamedTuple

import numpy as np

from . import _native as N


class Frame(NamedTuple):
    frame_id: int
    depth: np.ndarray  # (H, W) uint16, millimetres
    rgb: np.ndarray    # (H, W, 3) uint8, R, G, B, on the depth image's grid
    c2w: np.ndarray    # (4, 4) float32, camera-to-world, row-major


class FrameFolder:
    """Frames in the reference's folder layout under `root`."""

    def __init__(self, root):
        self.root = os.fspath(root)
        self.rgb_dir = os.path.join(self.root, "RGB")
        self.depth_dir = os.path.join(self.root, "depth")
        self.pose_dir = os.path.join(self.root, "tcw")

    def paths(self, frame_id):
        """(colour, depth, pose) paths of a frame; colour is <i>.jpg when it
        exists, else <i>.png (None when neither does)."""
        i = str(int(frame_id))
        colour = None
        for ext in (".jpg", ".png"):
            p = os.path.join(self.rgb_dir, i + ext)
            if os.path.exists(p):
                colour = p
                break
        return (colour, os.path.join(self.depth_dir, i + ".png"),
                os.path.join(self.pose_dir, i + ".txt"))

    def load(self, frame_id):
        """Frame `frame_id` (vh_load_frame), or None when its colour, depth
        or pose file is missing (the reference marks a frame without
        colour as missing, src/SaveFrame.cpp:166-169)."""
        L = N.lib()
        root = self.root.encode()
        i = int(frame_id)
        w, h = C.c_int32(), C.c_int32()
        s = L.vh_load_frame(root, i, None, 0, None, 0, None, C.byref(w), C.byref(h))
        if s == N.VH_ERR_IO:
            return None
        N.check(s)
        depth = np.empty((h.value, w.value), np.uint16)
        rgb = np.empty((h.value, w.value, 3), np.uint8)
        c2w = np.empty((4, 4), np.float32)
        s = L.vh_load_frame(root, i, depth.ctypes.data, depth.size, rgb.ctypes.data, rgb.size,
                            c2w.ctypes.data, C.byref(w), C.byref(h))
        if s == N.VH_ERR_IO:  # removed between the two calls
            return None
        N.check(s)
        return Frame(i, depth, rgb, c2w)

    def frames(self, start=0, step=20, stop=2025, max_missing=5, workers=0):
        """Frames start, start + step, ... below stop, as the reference's
        application loop visits them.  The walk ends once `max_missing`
        frames were missing; as in the reference, a frame that loads does
        not reset that count.

        workers > 0 decodes up to 2 * workers frames ahead on that many
        threads (the library's decoders run without the interpreter lock),
        so that decoding overlaps the caller's use of each frame; the frames
        and their order are the same as with workers = 0."""
        if step <= 0:
            raise ValueError("step must be positive")
        ids = range(int(start), int(stop), int(step))
        if workers <= 0:
            missing = 0
            for i in ids:
                if missing == max_missing:
                    return
                frame = self.load(i)
                if frame is None:
                    missing += 1
                    continue
                yield frame
            return
        with ThreadPoolExecutor(int(workers)) as pool:
            ahead = deque()
            todo = iter(ids)

            def top_up():
                while len(ahead) < 2 * workers:
                    i = next(todo, None)
                    if i is None:
                        return
                    ahead.append(pool.submit(self.load, i))

            try:
                top_up()
                missing = 0
                while ahead and missing < max_missing:
                    frame = ahead.popleft().result()
                    top_up()
                    if frame is None:
                        missing += 1
                        continue
                    yield frame
            finally:
                for f in ahead:  # loads past the end of the walk
                    f.cancel()
