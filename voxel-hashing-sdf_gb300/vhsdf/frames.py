"""RGB-D frames stored in the reference's folder layout, read into the
arrays Volume.integrate takes.

The reference's frame store (src/SaveFrame.cpp:44-52, 154-218) keeps frame
`i` of a sequence as

    <root>/RGB/<i>.jpg     colour (its writer stores <i>.png)
    <root>/depth/<i>.png   16-bit grayscale depth in millimetres
    <root>/tcw/<i>.txt     16 numbers: a row-major 4 x 4 camera-to-world pose

and its application loop (src/main.cpp:242-258) fuses frames 0, 20, 40, ...
below 2025, stopping once five of them were missing.  FrameFolder.load
returns one frame, FrameFolder.frames walks that schedule.  The decoding
and resizing are the library's (vh_decode_depth_png, vh_decode_colour_jpeg,
vh_decode_colour_png, vh_resize_colour); this module only finds files and
reads the pose text.

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
import os
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from typing import NamedTuple

import numpy as np

from . import _native as N
from .engine import decode_colour_jpeg, decode_colour_png, decode_depth_png, resize_colour

_PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"
_JPEG_SIGNATURE = b"\xff\xd8"


class Frame(NamedTuple):
    frame_id: int
    depth: np.ndarray  # (H, W) uint16, millimetres
    rgb: np.ndarray    # (H, W, 3) uint8, R, G, B, on the depth image's grid
    c2w: np.ndarray    # (4, 4) float32, camera-to-world, row-major


def read_pose(path):
    """The 4 x 4 camera-to-world pose of a tcw/<i>.txt file (16 numbers,
    row-major, separated by white space), last row set to (0, 0, 0, 1)."""
    with open(path) as f:
        values = f.read().split()
    if len(values) < 16:
        raise ValueError(f"{path}: a pose needs 16 numbers, found {len(values)}")
    m = np.array([float(v) for v in values[:16]], np.float32).reshape(4, 4)
    if not np.isfinite(m).all():
        raise ValueError(f"{path}: the pose is not finite")
    m[3] = (0.0, 0.0, 0.0, 1.0)
    return m


def decode_colour(data):
    """A colour file's bytes (JPEG or PNG) as (H, W, 3) uint8 RGB."""
    if bytes(data[:8]) == _PNG_SIGNATURE:
        return decode_colour_png(data)
    if bytes(data[:2]) == _JPEG_SIGNATURE:
        return decode_colour_jpeg(data)
    raise N.VhError(N.VH_ERR_UNSUPPORTED, "colour image is neither JPEG nor PNG")


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
        """Frame `frame_id`, or None when its colour, depth or pose file is
        missing (the reference marks a frame without colour as missing,
        src/SaveFrame.cpp:166-169)."""
        colour, depth_path, pose_path = self.paths(frame_id)
        if colour is None or not os.path.exists(depth_path) or not os.path.exists(pose_path):
            return None
        with open(depth_path, "rb") as f:
            depth = decode_depth_png(f.read())
        with open(colour, "rb") as f:
            rgb = decode_colour(f.read())
        if rgb.shape[:2] != depth.shape:
            rgb = resize_colour(rgb, depth.shape[1], depth.shape[0])
        return Frame(int(frame_id), depth, rgb, read_pose(pose_path))

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
