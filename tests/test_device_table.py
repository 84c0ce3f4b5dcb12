"""Device-side hash access (include/vhashing_device.cuh): the device members
of vhashing::HashTable - find / operator[] (include/vhashing.h:122-135),
Apply (:818-825) and Filter (:790-805) - as a caller's own kernels over the
addresses vh_get_device_table publishes.  tests/device_table_user.cu is
such a caller; its answers must equal the library's own calls on the same
volume (vh_find_keys, vh_export_blocks)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, REPO
from vhsdf import _native as N

USER_SRC = os.path.join(REPO, "tests", "device_table_user.cu")
NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    import shutil
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        pytest.skip("nvcc not available")
    return exe


def test_device_header_compiles(tmp_path):
    """The header compiles into a caller's translation unit for sm_103a
    (cross-compiled; no device needed)."""
    subprocess.run([nvcc(), "-std=c++17", "-O2", *NVCC_ARCH, "-Xcompiler", "-fPIC", "-I",
                    os.path.join(REPO, "include"), "-c", USER_SRC, "-o",
                    str(tmp_path / "user.o")], check=True, capture_output=True)


def test_device_header_hashes_like_the_engine():
    """The header restates the table's slot hash for callers' kernels; its
    finaliser constants and shifts must be the engine's (the GPU test below
    then checks lookups end to end)."""
    import re
    hdr = open(os.path.join(REPO, "include", "vhashing_device.cuh")).read()
    eng = open(os.path.join(PKG, "csrc", "vh_common.cuh")).read()

    def mix_body(text, name):
        body = re.search(name + r"\(unsigned long long z\) \{(.*?)\}", text, re.S).group(1)
        return re.findall(r"0x[0-9A-Fa-f]+ull|>> \d+", body)

    assert mix_body(hdr, "mix") == mix_body(eng, "mix64")
    assert len(mix_body(eng, "mix64")) == 5
    assert "<< 21" in hdr and "<< 42" in hdr and "0x1FFFFFull" in hdr


def test_device_table_host_checks():
    L = N.lib()
    t = N.VhDeviceTable()
    assert L.vh_get_device_table(None, C.byref(t)) == N.VH_ERR_INVALID_ARG
    assert C.sizeof(N.VhDeviceTable) == 72


@pytest.fixture(scope="module")
def user_lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("devtable") / "libdevtable_user.so"
    lib = os.path.join(PKG, "lib")
    subprocess.run([nvcc(), "-std=c++17", "-O2", *NVCC_ARCH, "-Xcompiler", "-fPIC", "-shared",
                    "-I", os.path.join(REPO, "include"), USER_SRC, "-L", lib, "-lvhsdf",
                    f"-Xlinker=-rpath,{lib}", "-o", str(out)], check=True, capture_output=True)
    U = C.CDLL(str(out))
    T = C.POINTER(N.VhDeviceTable)
    U.dt_lookup.argtypes = [T, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    U.dt_weight_sum.argtypes = [T, C.c_void_p]
    U.dt_filter.argtypes = [T, C.c_float, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]
    U.dt_cap_weights.argtypes = [T, C.c_float]
    return U


@pytest.mark.gpu
def test_device_members_match_the_library(gpu, user_lib):
    from helpers import small_scene, volume_for
    scene = small_scene()
    vol = volume_for(scene)
    for f in range(3):
        vol.integrate(*scene.render(f))
    t = vol.device_table()
    assert t.layout == N.VH_DEVICE_TABLE_LAYOUT and t.pool_capacity == vol.params.pool_blocks
    e = vol.export_blocks()
    present = e["xyz"]
    assert len(present) > 100
    missing = present[:50] + np.array([0, 0, 700], np.int32)
    out_of_range = np.array([[1 << 20, 0, 0], [0, -(1 << 20) - 1, 0]], np.int32)
    keys = np.ascontiguousarray(np.concatenate([present, missing, out_of_range]), np.int32)

    # find / operator[]
    ids = np.full(len(keys), -7, np.int32)
    sdf0 = np.empty(len(keys), np.float32)
    w511 = np.empty(len(keys), np.float32)
    assert user_lib.dt_lookup(C.byref(t), keys.ctypes.data, len(keys), ids.ctypes.data,
                              sdf0.ctypes.data, w511.ctypes.data) == 0
    assert np.array_equal(ids, vol.find_keys(keys))
    n = len(present)
    assert (ids[:n] >= 0).all() and (ids[n:] == -1).all()
    assert np.array_equal(sdf0[:n].view(np.uint32), e["sdf"][:, 0].view(np.uint32))
    assert np.array_equal(w511[:n].view(np.uint32), e["weight"][:, 511].view(np.uint32))

    # Apply
    tb = np.zeros(2, np.uint64)
    assert user_lib.dt_weight_sum(C.byref(t), tb.ctypes.data) == 0
    assert int(tb[1]) == n
    assert int(tb[0]) == int(e["weight"].astype(np.int64).sum())

    # Filter
    w_min = 3.0
    want = present[(e["weight"] >= w_min).any(axis=1)]
    assert 5 <= len(want) <= n
    cap = n
    fx = np.empty((cap, 3), np.int32)
    fi = np.empty(cap, np.int32)
    cnt = C.c_ulonglong()
    assert user_lib.dt_filter(C.byref(t), w_min, fx.ctypes.data, fi.ctypes.data, cap,
                              C.byref(cnt)) == 0
    m = cnt.value
    assert m == len(want)
    got = set(map(tuple, fx[:m].tolist()))
    assert got == set(map(tuple, want.tolist()))
    assert np.array_equal(fi[:m], vol.find_keys(np.ascontiguousarray(fx[:m])))
    # a capacity below the count: the count still reports every kept block
    assert user_lib.dt_filter(C.byref(t), w_min, fx.ctypes.data, fi.ctypes.data, 5,
                              C.byref(cnt)) == 0
    assert cnt.value == len(want)
    assert set(map(tuple, fx[:5].tolist())) <= got

    # ApplyVoxels writes voxel values in place
    assert user_lib.dt_cap_weights(C.byref(t), 2.0) == 0
    after = vol.export_blocks()
    order_a, order_b = np.lexsort(after["xyz"].T), np.lexsort(present.T)
    assert np.array_equal(after["xyz"][order_a], present[order_b])
    assert np.array_equal(after["weight"][order_a], np.minimum(e["weight"], 2.0)[order_b])
    assert np.array_equal(after["sdf"][order_a].view(np.uint32),
                          e["sdf"][order_b].view(np.uint32))
    vol.close()
