"""The Python wrapper checks every array the library would read by the
volume's parameters (image sizes, upstream gradients, imported blocks)
before it calls the C ABI.  Runs without a GPU: the volume is bound to a
recording stand-in for the library."""
import ctypes as C

import numpy as np
import pytest

from vhsdf import _native as N
from vhsdf.engine import Volume


class FakeLib:
    """Records C ABI calls; vh_block_list reports `frame_blocks` entries."""

    def __init__(self, frame_blocks=0):
        self.calls = []
        self.frame_blocks = frame_blocks

    def __getattr__(self, name):
        def call(*args):
            self.calls.append(name)
            if name == "vh_block_list" and args[-1] is not None:
                args[-1]._obj.value = self.frame_blocks
            return N.VH_OK
        return call


def fake_volume(width=64, height=48, frame_blocks=0):
    vol = Volume.__new__(Volume)
    p = N.VhParams()
    p.width, p.height, p.device = width, height, 0
    vol.params = p
    vol._L = FakeLib(frame_blocks)
    vol._h = C.c_void_p(1)
    return vol


def frame(w=64, h=48, dtype=np.uint16):
    return np.zeros((h, w), dtype), np.zeros((h, w, 3), np.uint8), np.eye(4, dtype=np.float32)


def test_frames_of_the_volume_size_reach_the_library():
    vol = fake_volume()
    vol.process_frame(*frame())
    vol.integrate(*frame(dtype=np.float32))
    assert vol._L.calls == ["vh_process_frame", "vh_integrate"]


@pytest.mark.parametrize("bad", ["depth", "rgb", "both_small", "f32_as_u16"])
def test_wrong_image_sizes_are_refused_before_the_call(bad):
    vol = fake_volume()
    d, c, p = frame()
    fmt = None
    if bad == "depth":
        d = np.zeros((47, 64), np.uint16)
    elif bad == "rgb":
        c = np.zeros((48, 64, 4), np.uint8)
    elif bad == "both_small":
        d, c, p = frame(32, 24)
    else:
        d = np.zeros((48, 64), np.float32)
        fmt = "u16"
    with pytest.raises(ValueError):
        vol.process_frame(d, c, p, depth_format=fmt)
    with pytest.raises(ValueError):
        vol.pose_refine(d if bad != "rgb" else np.zeros((1, 1), np.uint16), np.eye(4),
                        depth_format=fmt)
    assert vol._L.calls == []


def test_refinement_batches_check_every_image():
    vol = fake_volume()
    good = np.zeros((48, 64), np.uint16)
    vol.pose_refine_batch([good, good], np.stack([np.eye(4)] * 2))
    assert vol._L.calls == ["vh_pose_refine_batch"]
    with pytest.raises(ValueError):
        vol.pose_refine_batch([good, np.zeros((48, 63), np.uint16)], np.stack([np.eye(4)] * 2))


def test_vjp_gradient_must_cover_the_block_list():
    vol = fake_volume(frame_blocks=3)
    d = np.zeros((48, 64), np.float32)
    vol.integrate_vjp(d, np.eye(4), np.zeros((3, 512), np.float32))
    assert vol._L.calls[-1] == "vh_integrate_vjp"
    with pytest.raises(ValueError):
        vol.integrate_vjp(d, np.eye(4), np.zeros((2, 512), np.float32))


def test_imported_blocks_must_match_their_keys():
    vol = fake_volume()
    xyz = np.zeros((2, 3), np.int32)
    sdf, w = np.zeros((2, 512), np.float32), np.ones((2, 512), np.float32)
    rgb = np.zeros((2, 512, 3), np.uint8)
    vol.import_blocks(xyz, sdf, w, rgb)
    assert vol._L.calls == ["vh_import_blocks"]
    for args in ((xyz, sdf[:1], w, rgb), (xyz, sdf, w[:, :100], rgb), (xyz, sdf, w, rgb[:, :, :2])):
        with pytest.raises(ValueError):
            vol.import_blocks(*args)
    assert vol._L.calls == ["vh_import_blocks"]
