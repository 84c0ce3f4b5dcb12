"""vh_find_keys_noalloc: the key lookup for callers that must not allocate
device memory (a latency-bound loop that cannot take cudaFree's device-wide
synchronisation, or a plugin whose host framework owns all device memory).
Through the C ABI, its answers must equal vh_find_keys' on the same keys,
on two calls in a row (the shared scratch array keeps the previous call's
contents)."""
import ctypes as C

import numpy as np
import pytest

from helpers import small_scene, volume_for
from vhsdf import _native as N

pytestmark = pytest.mark.gpu


def find_existing(vol, keys):
    out = np.empty(len(keys), np.int32)
    st = N.lib().vh_find_keys(vol._h, keys.ctypes.data, len(keys), out.ctypes.data,
                              N.VH_MEM_HOST)
    assert st == N.VH_OK
    return out


def find_noalloc(vol, keys):
    out = np.full(len(keys), -7, np.int32)
    st = N.lib().vh_find_keys_noalloc(vol._h, keys.ctypes.data, len(keys), out.ctypes.data)
    assert st == N.VH_OK, N.lib().vh_last_error(vol._h)
    return out


def test_noalloc_lookup_matches_find_keys(gpu):
    scene = small_scene()
    vol = volume_for(scene)
    for f in range(3):
        vol.integrate(*scene.render(f))
    present = vol.export_blocks()["xyz"]
    rng = np.random.default_rng(3)
    missing = present + np.array([0, 0, 1000], np.int32)
    out_of_range = np.array([[1 << 20, 0, 0], [0, -(1 << 20) - 1, 5]], np.int32)
    first = np.ascontiguousarray(np.concatenate([present, missing, out_of_range]), np.int32)
    rng.shuffle(first)
    # a second, smaller call: stale answers from the first would show up here
    second = np.ascontiguousarray(np.concatenate([missing[:50], present[::3]]), np.int32)
    rng.shuffle(second)
    for keys in (first, second):
        want = find_existing(vol, keys)
        got = find_noalloc(vol, keys)
        assert np.array_equal(got, want)
    assert np.all(find_noalloc(vol, present) >= 0)
    assert np.all(find_noalloc(vol, missing) == -1)


def test_noalloc_rejects_oversized_calls(gpu):
    scene = small_scene()
    vol = volume_for(scene)
    n = 65536 + 1
    keys = np.zeros((n, 3), np.int32)
    out = np.empty(n, np.int32)
    st = N.lib().vh_find_keys_noalloc(vol._h, keys.ctypes.data, n, out.ctypes.data)
    assert st == N.VH_ERR_CAPACITY
    assert b"VH_FIND_NOALLOC_MAX_KEYS" in N.lib().vh_last_error(vol._h)
    assert N.lib().vh_find_keys_noalloc(vol._h, keys.ctypes.data, 0, out.ctypes.data) == N.VH_OK
    assert N.lib().vh_find_keys_noalloc(None, keys.ctypes.data, 1, out.ctypes.data) == \
        N.VH_ERR_INVALID_ARG
