"""The C ABI library loads, exports every declared entry point and validates
parameters on the host (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from conftest import REPO, cuda_available


def declared_functions():
    text = open(os.path.join(REPO, "include", "vhsdf.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vh_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    from vhsdf import _native as N
    L = C.CDLL(N.ENGINE_PATH)
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(N.SIGNATURES), "ctypes binding out of sync with the header"


def test_params_default_and_validate():
    from vhsdf import _native as N
    L = N.lib()
    p = N.VhParams()
    assert L.vh_params_default(C.byref(p)) == N.VH_OK
    assert (p.width, p.height, p.fx, p.cx) == (640, 480, 577.0, 320.0)
    assert abs(p.voxel_size - 0.036) < 1e-7 and abs(p.trunc - 0.18) < 1e-7
    assert L.vh_params_validate(C.byref(p)) == N.VH_OK
    bad = [("width", 0), ("fx", -1.0), ("voxel_size", 0.0), ("table_log2", 40),
           ("max_probe", 0), ("pool_blocks", 0), ("flags", 0x80)]
    for field, val in bad:
        q = N.VhParams()
        L.vh_params_default(C.byref(q))
        setattr(q, field, val)
        assert L.vh_params_validate(C.byref(q)) != N.VH_OK, field
    q = N.VhParams()
    L.vh_params_default(C.byref(q))
    q.flags = N.VH_FLAG_SYNC | N.VH_FLAG_BATCH_FUSED  # the batch form flag is a known flag
    assert L.vh_params_validate(C.byref(q)) == N.VH_OK
    q = N.VhParams()
    L.vh_params_default(C.byref(q))
    q.trunc = float("nan")
    assert L.vh_params_validate(C.byref(q)) == N.VH_ERR_NOT_FINITE
    assert L.vh_params_validate(None) == N.VH_ERR_INVALID_ARG


def test_status_strings_and_null_handles():
    from vhsdf import _native as N
    L = N.lib()
    for s in range(12):
        assert L.vh_status_string(s)
    assert L.vh_destroy(None) == N.VH_ERR_INVALID_ARG
    assert L.vh_sync(None) == N.VH_ERR_INVALID_ARG
    assert L.vh_render(None) == N.VH_ERR_UNSUPPORTED
    assert L.vh_last_error(None) == b"null handle"
    nv, nf = C.c_int64(-1), C.c_int64(-1)
    assert L.vh_process_frame_indexed(None, None, N.VH_DEPTH_U16_MM, None, None, N.VH_MEM_HOST,
                                      None, 0, None, 0, C.byref(nv),
                                      C.byref(nf)) == N.VH_ERR_INVALID_ARG
    t = N.VhDeviceTable()
    assert L.vh_get_device_table(None, C.byref(t)) == N.VH_ERR_INVALID_ARG
    # argument checks come before any device work
    poses = (C.c_float * 16)()
    out = (C.c_float * 16)()
    tab = (C.c_void_p * 1)(None)
    assert L.vh_pose_refine_batch(None, C.cast(tab, C.c_void_p), N.VH_DEPTH_U16_MM,
                                  N.VH_MEM_HOST, 1, poses, 20, 1, out, None) == N.VH_ERR_INVALID_ARG
    assert L.vh_pose_refine(None, None, N.VH_DEPTH_U16_MM, N.VH_MEM_HOST, poses, 20, 1,
                            N.VH_REFINE_ADJOINT, out, None) == N.VH_ERR_INVALID_ARG


@pytest.mark.skipif(cuda_available(), reason="checks the no-device path")
def test_create_without_device_reports_no_device():
    from vhsdf import _native as N
    L = N.lib()
    p = N.VhParams()
    L.vh_params_default(C.byref(p))
    h = C.c_void_p()
    assert L.vh_create(C.byref(p), C.byref(h)) == N.VH_ERR_NO_DEVICE
    assert not h.value


def test_missing_library_fails_loudly(monkeypatch):
    from vhsdf import _native as N
    monkeypatch.setattr(N, "_lib", None)
    monkeypatch.setattr(N, "ENGINE_PATH", "/nonexistent/libvhsdf.so")
    with pytest.raises(ImportError):
        N.lib()


def test_batch_rejects_unsupported_parameters_on_the_host():
    from vhsdf import Batch, VhError, _native as N
    with pytest.raises(VhError) as err:
        Batch([dict(width=64, height=48), dict(width=64, height=48, flags=N.VH_FLAG_DEPTH_FILTER)])
    assert err.value.status == N.VH_ERR_UNSUPPORTED
    with pytest.raises(VhError) as err:
        Batch([dict(width=64, height=48, voxel_size=0.0)])
    assert err.value.status == N.VH_ERR_INVALID_ARG


def test_tuning_variant_counts():
    """Launch-shape counts are host facts (no device call): 6 integration
    shapes and 3 marching-cubes shapes, and both pointers may be NULL."""
    from vhsdf import Volume
    from vhsdf import _native as N
    assert Volume.tuning_variants() == (6, 3)
    N.lib().vh_tuning_variants(None, None)


def test_log_callback_receives_create_failures():
    """vh_set_log_callback: a vh_create that fails before a handle exists
    (device index 99: no device here, out of range on a GPU machine) reports
    its reason to the callback; removing the callback stops the messages."""
    import vhsdf
    from vhsdf import _native as N
    got = []
    vhsdf.set_log_callback(lambda level, msg: got.append((level, msg)))
    try:
        L = N.lib()
        p = N.VhParams()
        L.vh_params_default(C.byref(p))
        p.device = 99
        h = C.c_void_p()
        st = L.vh_create(C.byref(p), C.byref(h))
        assert st in (N.VH_ERR_NO_DEVICE, N.VH_ERR_INVALID_ARG)
        assert len(got) == 1 and got[0][0] == N.VH_LOG_ERROR
        assert "vh_create" in got[0][1] and ("no CUDA device" in got[0][1] or "out of range" in got[0][1])
        q = N.VhParams()
        L.vh_params_default(C.byref(q))
        q.voxel_size = 0.0
        assert L.vh_create(C.byref(q), C.byref(h)) != N.VH_OK
        assert len(got) == 2 and "invalid parameters" in got[1][1]
    finally:
        vhsdf.set_log_callback(None)
    L.vh_create(C.byref(p), C.byref(h))
    assert len(got) == 2


def test_checked_build_loads_and_reports_its_flag():
    """Both builds export every declared entry point; only the checked one
    reports VH_BUILD_CHECKED."""
    from vhsdf import _native as N
    plain = C.CDLL(os.path.join(N.LIB_DIR, "libvhsdf.so"))
    checked = C.CDLL(os.path.join(N.LIB_DIR, "libvhsdf_checked.so"))
    for L in (plain, checked):
        L.vh_build_flags.restype = C.c_uint32
        for n in declared_functions():
            assert hasattr(L, n), n
    assert plain.vh_build_flags() == 0
    assert checked.vh_build_flags() == N.VH_BUILD_CHECKED
    assert plain.vh_status_string(N.VH_ERR_CHECK)
