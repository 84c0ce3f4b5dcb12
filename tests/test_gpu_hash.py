"""The hash surface (vhashing::HashTable) on the GPU: set semantics against
the reference's recorded op sequence, duplicates, capacity limits."""
import json
import os

import numpy as np
import pytest

from conftest import REPO
from helpers import key_set, small_scene, volume_for
from vhsdf import VhError, Volume, _native as N

pytestmark = pytest.mark.gpu


def hash_volume(**kw):
    p = dict(width=64, height=48, voxel_size=0.01, trunc=0.04, table_log2=12,
             pool_blocks=2048, max_frame_blocks=4096, max_triangles=1024)
    p.update(kw)
    return Volume(**p)


def test_reference_op_sequence(gpu):
    """Replays the insert / erase / find sequence recorded from the
    reference's host HashTable.  The engine answers every op like a set; the
    reference differs only on the key it loses (see test_golden)."""
    with open(os.path.join(REPO, "tests", "golden", "ref_golden.json")) as f:
        ops = np.array(json.load(f)["hash_ops"], np.int64).reshape(-1, 5)
    from test_golden import REFERENCE_LOST_KEY_OPS
    vol = hash_volume()
    mismatches = []
    for i, (op, x, y, z, res) in enumerate(ops):
        k = np.array([[x, y, z]], np.int32)
        if op == 0:
            was = vol.find_keys(k)[0] >= 0
            vol.alloc_keys(k)
            got = int(not was)
        elif op == 1:
            got = vol.erase_keys(k)
        else:
            got = int(vol.find_keys(k)[0] >= 0)
        if got != res:
            mismatches.append(i)
    assert mismatches == REFERENCE_LOST_KEY_OPS


def test_bulk_alloc_with_duplicates(gpu):
    rng = np.random.default_rng(1)
    keys = rng.integers(-40, 40, size=(200_000, 3)).astype(np.int32)
    vol = hash_volume(table_log2=20, pool_blocks=600_000, max_frame_blocks=600_000)
    vol.clear_block_list()
    vol.alloc_keys(keys)
    uniq = np.unique(keys, axis=0)
    st = vol.stats()
    assert st["blocks_allocated"] == len(uniq)
    ids = vol.find_keys(uniq)
    assert np.all(ids >= 0) and len(np.unique(ids)) == len(uniq)
    assert key_set(vol.block_list()) == key_set(uniq)
    missing = np.array([[100, 100, 100], [-100, 5, 5]], np.int32)
    assert np.all(vol.find_keys(missing) == -1)
    # the same keys again create nothing
    vol.alloc_keys(keys[:1000])
    assert vol.stats()["blocks_allocated"] == len(uniq)


def test_device_key_buffers(gpu):
    import torch
    vol = hash_volume()
    keys = torch.tensor([[1, 2, 3], [4, 5, 6], [1, 2, 3]], dtype=torch.int32, device="cuda")
    vol.alloc_keys(keys)
    ids = vol.find_keys(keys)
    assert ids.is_cuda and ids[0].item() == ids[2].item() >= 0 and ids[1].item() >= 0
    assert vol.stats()["blocks_allocated"] == 2


def test_table_full_reports_error_without_hanging(gpu):
    vol = hash_volume(table_log2=8, max_probe=8, pool_blocks=4096)
    keys = np.stack(np.meshgrid(np.arange(20), np.arange(20), np.arange(2), indexing="ij"),
                    -1).reshape(-1, 3).astype(np.int32)
    with pytest.raises(VhError) as e:
        vol.alloc_keys(keys)
    assert e.value.status == N.VH_ERR_TABLE_FULL
    # the handle stays usable
    assert vol.find_keys(keys[:1])[0] >= -1
    vol.sync()


def test_pool_full_reports_error(gpu):
    vol = hash_volume(pool_blocks=100)
    keys = np.stack([np.arange(300), np.zeros(300), np.zeros(300)], -1).astype(np.int32)
    with pytest.raises(VhError) as e:
        vol.alloc_keys(keys)
    assert e.value.status == N.VH_ERR_POOL_FULL
    assert vol.stats()["blocks_allocated"] == 100


def test_out_of_range_keys(gpu):
    vol = hash_volume()
    with pytest.raises(VhError) as e:
        vol.alloc_keys(np.array([[1 << 20, 0, 0]], np.int32))
    assert e.value.status == N.VH_ERR_OUT_OF_RANGE
    assert vol.find_keys(np.array([[1 << 20, 0, 0]], np.int32))[0] == -1
    vol.alloc_keys(np.array([[(1 << 20) - 1, -(1 << 20), 0]], np.int32))
    assert vol.find_keys(np.array([[(1 << 20) - 1, -(1 << 20), 0]], np.int32))[0] >= 0


def test_erase_recycles_zeroed_blocks(gpu):
    scene = small_scene()
    vol = volume_for(scene, pool_blocks=1 << 15)
    for f in range(3):
        vol.integrate(*scene.render(f))
    e = vol.export_blocks()
    n0 = len(e["xyz"])
    victims = e["xyz"][: n0 // 2]
    assert vol.erase_keys(victims) == len(victims)
    assert vol.erase_keys(victims) == 0
    st = vol.stats()
    assert st["blocks_allocated"] == n0 - len(victims)
    assert st["tombstones"] == len(victims)
    assert np.all(vol.find_keys(victims) == -1)
    fresh = victims + np.array([1000, 0, 0], np.int32)
    vol.alloc_keys(fresh)
    e2 = vol.export_blocks()
    assert len(e2["xyz"]) == n0
    new = np.isin(e2["xyz"][:, 0], fresh[:, 0]) & (e2["xyz"][:, 0] >= 900)
    assert new.sum() == len(fresh)
    assert np.all(e2["sdf"][new] == 0) and np.all(e2["weight"][new] == 0)
    assert np.all(e2["rgb"][new] == 0)
    # recycled ids come from the erased ones: the pool did not grow
    assert vol.stats()["blocks_allocated"] == n0


def test_block_list_and_clear(gpu):
    vol = hash_volume()
    vol.alloc_keys(np.array([[0, 0, 0], [1, 0, 0]], np.int32))
    assert key_set(vol.block_list()) == {(0, 0, 0), (1, 0, 0)}
    vol.clear_block_list()
    assert len(vol.block_list()) == 0
    vol.alloc_keys(np.array([[1, 0, 0], [2, 0, 0]], np.int32))
    assert key_set(vol.block_list()) == {(1, 0, 0), (2, 0, 0)}
    assert vol.stats()["blocks_allocated"] == 3
