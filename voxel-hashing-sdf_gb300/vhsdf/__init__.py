"""vhsdf - GB300-native voxel-hashing TSDF engine (Python front end).

The compute path is the native library lib/libvhsdf.so (CUDA for sm_103a
behind a C ABI, include/vhsdf.h); this package only marshals arguments.
"""
from ._native import VhError, BLOCK_EDGE, BLOCK_VOXELS, set_log_callback  # noqa: F401
from .engine import (Volume, block_hash_ref, decode_colour_jpeg,  # noqa: F401
                     decode_colour_png, decode_depth_png, resize_colour)
from .frames import Frame, FrameFolder  # noqa: F401
from .batch import Batch  # noqa: F401
from .generator import GpuTsdfGenerator, HashTable  # noqa: F401
from . import synth  # noqa: F401
