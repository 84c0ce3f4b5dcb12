"""ctypes binding of the engine's C ABI (include/vhsdf.h).

The engine library must exist: there is no fallback.  Build it with
``python voxel-hashing-sdf_gb300/build_native.py`` (or ``__graft_entry__.build()``).
"""
import ctypes as C
import os

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(PKG, "lib")
# VHSDF_CHECKED=1 selects the build whose per-frame kernels check every index
# they derive (errors as VH_ERR_CHECK instead of faults), for debugging.
ENGINE_PATH = os.path.join(LIB_DIR, "libvhsdf_checked.so" if os.environ.get("VHSDF_CHECKED") == "1"
                           else "libvhsdf.so")
SYNTH_PATH = os.path.join(LIB_DIR, "libvhsynth.so")

VH_OK = 0
VH_ERR_INVALID_ARG = 1
VH_ERR_CUDA = 2
VH_ERR_TABLE_FULL = 3
VH_ERR_POOL_FULL = 4
VH_ERR_RETRY_EXHAUSTED = 5
VH_ERR_NOT_FINITE = 6
VH_ERR_UNSUPPORTED = 7
VH_ERR_OUT_OF_RANGE = 8
VH_ERR_CAPACITY = 9
VH_ERR_IO = 10
VH_ERR_NO_DEVICE = 11
VH_ERR_CHECK = 12
VH_BUILD_CHECKED = 1

VH_DEPTH_U16_MM = 0
VH_DEPTH_F32_M = 1
VH_MEM_HOST = 0
VH_MEM_DEVICE = 1
VH_SCOPE_FRAME = 0
VH_SCOPE_ALL = 1
VH_FLAG_SYNC = 0x1
VH_FLAG_NO_GRAPH = 0x2
VH_FLAG_PROFILE = 0x4
VH_FLAG_DEPTH_FILTER = 0x8
VH_FLAG_BATCH_FUSED = 0x10
VH_REFINE_BATCH_MAX = 256
VH_REFINE_ADJOINT = 0
VH_REFINE_FD = 1
BLOCK_EDGE = 8
BLOCK_VOXELS = 512


class VhParams(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32),
        ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
        ("min_depth", C.c_float), ("max_depth", C.c_float), ("depth_scale", C.c_float),
        ("voxel_size", C.c_float), ("trunc", C.c_float), ("mc_min_weight", C.c_float),
        ("table_log2", C.c_int32), ("max_probe", C.c_int32),
        ("pool_blocks", C.c_int64), ("max_frame_blocks", C.c_int64),
        ("max_triangles", C.c_int64),
        ("flags", C.c_uint32), ("device", C.c_int32),
    ]


class VhStats(C.Structure):
    _fields_ = [
        ("frames", C.c_int64), ("blocks_allocated", C.c_int64), ("frame_blocks", C.c_int64),
        ("new_blocks", C.c_int64), ("voxels_updated", C.c_int64), ("triangles", C.c_int64),
        ("pool_capacity", C.c_int64), ("table_slots", C.c_int64), ("tombstones", C.c_int64),
        ("device_error", C.c_uint32), ("frame_kernels", C.c_uint32),
        ("ms_allocate", C.c_float), ("ms_integrate", C.c_float), ("ms_extract", C.c_float),
        ("ms_frame", C.c_float),
    ]


class VhTuning(C.Structure):
    _fields_ = [("integrate_variant", C.c_int32), ("integrate_ctas_per_sm", C.c_int32),
                ("mc_ctas_per_sm", C.c_int32), ("mc_variant", C.c_int32)]


class VhRefineStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("valid_pixels", C.c_int32),
                ("initial_rmse", C.c_float), ("final_rmse", C.c_float), ("ms", C.c_float),
                ("ms_steps", C.c_float)]


class VhMeshView(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("num_triangles", C.c_int64),
                ("voxel_size", C.c_float)]


class VhDeviceTable(C.Structure):
    _fields_ = [("layout", C.c_uint32), ("slot_mask", C.c_uint32), ("max_probe", C.c_int32),
                ("key_bias", C.c_int32), ("slots", C.c_void_p), ("pool", C.c_void_p),
                ("block_keys", C.c_void_p), ("pool_top", C.c_void_p),
                ("pool_capacity", C.c_int64), ("voxel_size", C.c_float), ("device", C.c_int32),
                ("stream", C.c_void_p)]


VH_DEVICE_TABLE_LAYOUT = 1

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
PI64 = C.POINTER(C.c_int64)

# name -> (restype, argtypes); mirrors include/vhsdf.h
SIGNATURES = {
    "vh_params_default": (I32, [C.POINTER(VhParams)]),
    "vh_params_validate": (I32, [C.POINTER(VhParams)]),
    "vh_status_string": (C.c_char_p, [I32]),
    "vh_create": (I32, [C.POINTER(VhParams), C.POINTER(P)]),
    "vh_destroy": (I32, [P]),
    "vh_reset": (I32, [P]),
    "vh_set_stream": (I32, [P, P]),
    "vh_sync": (I32, [P]),
    "vh_last_error": (C.c_char_p, [P]),
    "vh_integrate": (I32, [P, P, I32, P, P, I32]),
    "vh_extract": (I32, [P, I32, C.POINTER(VhMeshView)]),
    "vh_process_frame": (I32, [P, P, I32, P, P, I32, C.POINTER(VhMeshView)]),
    "vh_process_frame_mesh": (I32, [P, P, I32, P, P, I32, P, I64, PI64]),
    "vh_process_frame_indexed": (I32, [P, P, I32, P, P, I32, P, I64, P, I64, PI64, PI64]),
    "vh_copy_mesh": (I32, [P, P, P, I64, PI64]),
    "vh_save_ply": (I32, [P, C.c_char_p, I32]),
    "vh_render": (I32, [P]),
    "vh_alloc_keys": (I32, [P, P, I64, I32]),
    "vh_find_keys": (I32, [P, P, I64, P, I32]),
    "vh_find_keys_noalloc": (I32, [P, P, I64, P]),
    "vh_erase_keys": (I32, [P, P, I64, PI64, I32]),
    "vh_clear_block_list": (I32, [P]),
    "vh_block_list": (I32, [P, P, I64, PI64]),
    "vh_block_hash_ref": (C.c_uint64, [I32, I32, I32]),
    "vh_get_device_table": (I32, [P, C.POINTER(VhDeviceTable)]),
    "vh_mc_tables": (I32, [P, P, P]),
    "vh_export_blocks": (I32, [P, P, P, P, P, I64, PI64]),
    "vh_import_blocks": (I32, [P, P, P, P, P, I64]),
    "vh_save": (I32, [P, C.c_char_p]),
    "vh_load": (I32, [P, C.c_char_p]),
    "vh_get_stats": (I32, [P, C.POINTER(VhStats)]),
    "vh_get_tuning": (I32, [P, C.POINTER(VhTuning)]),
    "vh_set_tuning": (I32, [P, C.POINTER(VhTuning)]),
    "vh_tuning_variants": (None, [C.POINTER(I32), C.POINTER(I32)]),
    "vh_set_log_callback": (None, [C.c_void_p, C.c_void_p]),
    "vh_build_flags": (C.c_uint32, []),
    "vh_autotune": (I32, [P, P, I32, P, P, I32, C.POINTER(VhTuning)]),
    "vh_sdf_sample": (I32, [P, P, I64, P, P, P, I32]),
    "vh_pose_normal_equations": (I32, [P, P, I32, I32, P, I32, I32, P]),
    "vh_pose_refine": (I32, [P, P, I32, I32, P, I32, I32, I32, P, C.POINTER(VhRefineStats)]),
    "vh_pose_refine_batch": (I32, [P, P, I32, I32, I32, P, I32, I32, P, C.POINTER(VhRefineStats)]),
    "vh_integrate_vjp": (I32, [P, P, I32, P, P, P, P, I32]),
    "vh_raycast": (I32, [P, P, P, P, P, I32]),
    "vh_filter_depth": (I32, [P, P, I32, P, I32]),
    "vh_decode_depth_png": (I32, [P, I64, P, I64, C.POINTER(I32), C.POINTER(I32)]),
    "vh_decode_colour_png": (I32, [P, I64, P, I64, C.POINTER(I32), C.POINTER(I32)]),
    "vh_resize_colour": (I32, [P, I32, I32, P, I32, I32]),
    "vh_decode_colour_jpeg": (I32, [P, I64, P, I64, C.POINTER(I32), C.POINTER(I32)]),
    "vh_load_frame": (I32, [C.c_char_p, I32, P, I64, P, I64, P, C.POINTER(I32), C.POINTER(I32)]),
    "vh_stream_out": (I32, [P, P, C.c_float, PI64]),
    "vh_stream_in": (I32, [P, P, C.c_float, PI64]),
    "vh_evict_async": (I32, [P, P, C.c_float]),
    "vh_host_blocks": (I64, [P]),
    "vh_compact_table": (I32, [P]),
    "vh_mesh_indexed": (I32, [P, P, P, I64, P, I64, PI64, PI64]),
    "vh_batch_create": (I32, [C.POINTER(VhParams), I32, C.POINTER(P)]),
    "vh_batch_destroy": (I32, [P]),
    "vh_batch_size": (I32, [P]),
    "vh_batch_scene": (P, [P, I32]),
    "vh_batch_process": (I32, [P, P, I32, P, P, I32, I32]),
    "vh_batch_sync": (I32, [P, P, C.POINTER(VhStats)]),
}

_lib = None
_synth = None


class VhError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


def lib():
    """The loaded engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(ENGINE_PATH):
            raise ImportError(f"vhsdf engine library missing: {ENGINE_PATH} (run build_native.py)")
        L = C.CDLL(ENGINE_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def synth_lib():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_PATH):
            raise ImportError(f"synthetic scene library missing: {SYNTH_PATH}")
        L = C.CDLL(SYNTH_PATH)
        L.vhs_create.restype = C.c_void_p
        L.vhs_create.argtypes = [I32, C.c_uint64, I32, I32, C.c_float, C.c_float, C.c_float,
                                 C.c_float, I32]
        L.vhs_destroy.argtypes = [P]
        L.vhs_num_frames.restype = I32
        L.vhs_num_frames.argtypes = [P]
        L.vhs_num_objects.restype = I32
        L.vhs_num_objects.argtypes = [P]
        L.vhs_bounds.argtypes = [P, P]
        L.vhs_render.restype = I32
        L.vhs_render.argtypes = [P, I32, P, P, P, I32]
        _synth = L
    return _synth


def check(status, handle=None):
    if status != VH_OK:
        L = lib()
        msg = L.vh_status_string(status).decode()
        if handle:
            detail = L.vh_last_error(handle)
            if detail:
                msg = f"{msg}: {detail.decode()}"
        raise VhError(status, msg)


VH_LOG_ERROR = 2
LOG_FN = C.CFUNCTYPE(None, C.c_int32, C.c_char_p, C.c_void_p)
_log_cb = None  # the installed ctypes callback (kept alive while installed)


def set_log_callback(fn):
    """Installs fn(level, message) as the library's log sink
    (vh_set_log_callback); None removes it.  fn runs on the thread that hit
    the error and must not call back into the library."""
    global _log_cb
    L = lib()
    if fn is None:
        L.vh_set_log_callback(None, None)
        _log_cb = None
        return
    cb = LOG_FN(lambda level, msg, user: fn(int(level), msg.decode(errors="replace")))
    L.vh_set_log_callback(C.cast(cb, C.c_void_p), None)
    _log_cb = cb
