"""Batched scenes on the GPU: a batch of uneven scenes stepped together must
leave every scene exactly as the same frames do through its own handle
(block set, voxels and the per-frame meshes bit for bit), and one scene is
checked against the FP32 oracle directly."""
import numpy as np
import pytest

from helpers import assert_same_blocks, oracle_for, sort_rows, tri_rows
from vhsdf import Batch, VhError, Volume, synth
from vhsdf import _native as N

pytestmark = pytest.mark.gpu

# (kind, seed, width, height, voxel, table_log2, frames): uneven sizes,
# pixel counts that are not multiples of 32, scenes that stop early
SCENES = [
    (1, 0, 160, 120, 0.02, 16, 6),
    (3, 101, 200, 150, 0.015, 17, 4),
    (3, 102, 96, 72, 0.03, 14, 6),
    (2, 2, 320, 240, 0.01, 18, 3),
    (3, 103, 130, 98, 0.025, 15, 5),
]


def scene_params(kind, seed, w, h, voxel, tlog, frames):
    sc = synth.Scene(kind=kind, seed=seed, num_frames=frames, width=w, height=h)
    prm = dict(width=w, height=h, fx=sc.fx, fy=sc.fy, cx=sc.cx, cy=sc.cy, min_depth=0.1,
               max_depth=4.5, voxel_size=voxel, trunc=4 * voxel, table_log2=tlog,
               pool_blocks=1 << (tlog - 1), max_frame_blocks=1 << (tlog - 1),
               max_triangles=1 << 20)
    return sc, prm


# Both step forms: a launch per stage and scene group, and one persistent
# launch over every stage of every scene (VH_FLAG_BATCH_FUSED).
MODES = {"staged": 0, "fused": N.VH_FLAG_BATCH_FUSED}


@pytest.fixture(scope="module", params=sorted(MODES))
def runs(gpu, request):
    scenes = [scene_params(*s) for s in SCENES]
    frames = [[sc.render(f) for f in range(s[-1])] for (sc, _), s in zip(scenes, SCENES)]
    steps = max(s[-1] for s in SCENES)
    flags = [dict(prm, flags=N.VH_FLAG_SYNC | MODES[request.param]) for _, prm in scenes]
    batch = Batch(flags)
    batch_meshes = [[] for _ in SCENES]
    for k in range(steps):
        step = [fr[k] if k < len(fr) else None for fr in frames]
        batch.process(step, with_mesh=True)
        status, stats = batch.sync()
        assert all(s == 0 for s in status), status
        for i, fr in enumerate(step):
            if fr is not None:
                batch_meshes[i].append(batch.scene(i).mesh())
                assert stats[i]["frames"] == k + 1
    singles, single_meshes = [], []
    for (sc, prm), fr in zip(scenes, frames):
        vol = Volume(**prm)
        ms = []
        for d, c, p in fr:
            vol.process_frame(d, c, p)
            ms.append(vol.mesh())
        singles.append(vol)
        single_meshes.append(ms)
    return scenes, frames, batch, batch_meshes, singles, single_meshes


def test_blocks_equal_single_scene_runs(runs):
    scenes, frames, batch, _, singles, _ = runs
    for i in range(len(SCENES)):
        assert_same_blocks(batch.scene(i).export_blocks(), singles[i].export_blocks())


def test_frame_meshes_equal_single_scene_runs(runs):
    _, frames, _, batch_meshes, _, single_meshes = runs
    for i in range(len(SCENES)):
        assert len(batch_meshes[i]) == len(single_meshes[i]) == len(frames[i])
        for (bx, bc), (sx, scol) in zip(batch_meshes[i], single_meshes[i]):
            assert len(bx) == len(sx)
            assert np.array_equal(sort_rows(tri_rows(bx, bc)), sort_rows(tri_rows(sx, scol)))


def test_one_scene_against_fp32_oracle(runs):
    scenes, frames, batch, _, _, _ = runs
    i = 1
    vol = batch.scene(i)
    orc = oracle_for(vol, 32)
    for d, c, p in frames[i]:
        orc.integrate(d, c, p)
    assert_same_blocks(vol.export_blocks(), orc.export())


def test_scene_handles_stay_usable(runs):
    """After batched steps a scene is an ordinary handle: full-volume
    extraction and stats work and agree with the single-scene run."""
    _, _, batch, _, singles, _ = runs
    for i in (0, 3):
        vol = batch.scene(i)
        vol.extract("all")
        singles[i].extract("all")
        bx, bc = vol.mesh()
        sx, scol = singles[i].mesh()
        assert np.array_equal(sort_rows(tri_rows(bx, bc)), sort_rows(tri_rows(sx, scol)))
        assert vol.stats()["blocks_allocated"] == singles[i].stats()["blocks_allocated"]


@pytest.mark.parametrize("mode", sorted(MODES))
def test_pool_overflow_is_reported_per_scene(gpu, mode):
    sc_a, prm_a = scene_params(1, 0, 160, 120, 0.02, 16, 2)
    sc_b, prm_b = scene_params(3, 104, 160, 120, 0.02, 16, 2)
    prm_a["flags"] = N.VH_FLAG_SYNC | MODES[mode]
    prm_b["pool_blocks"] = 64  # far too small
    batch = Batch([prm_a, prm_b])
    with pytest.raises(VhError) as err:  # synchronous handles: the step reports the first error
        batch.process([sc_a.render(0), sc_b.render(0)], with_mesh=False)
    assert err.value.status == 4  # VH_ERR_POOL_FULL
    status, stats = batch.sync()
    assert status[0] == 0
    assert status[1] != 0 and stats[1]["device_error"] != 0
    # the error was cleared; the healthy scene keeps going
    batch.process([sc_a.render(1), None])
    status, _ = batch.sync()
    assert status == [0, 0]
    batch.close()


def test_retuning_scene_zero_rebuilds_the_batch_graph(gpu):
    specs = [scene_params(*s) for s in SCENES[:3]]
    frames = [[sc.render(f) for f in range(3)] for sc, _ in specs]
    batch = Batch([prm for _, prm in specs])
    singles = [Volume(**prm) for _, prm in specs]
    for k in range(3):
        if k == 1:
            batch.scene(0).set_tuning(1, 2, 3, 1)  # other launch shapes from now on
        batch.process([fr[k] for fr in frames], with_mesh=True)
        status, _ = batch.sync()
        assert status == [0, 0, 0]
        for v, fr in zip(singles, frames):
            v.process_frame(*fr[k])
    for i, v in enumerate(singles):
        assert_same_blocks(batch.scene(i).export_blocks(), v.export_blocks())
    batch.close()


def test_fused_steps_without_meshes_and_with_idle_scenes(gpu):
    """The persistent step without extraction, with scenes that have no
    frame in some steps and a scene whose frames miss the volume entirely
    (no valid depth: an empty frame list), equals per-scene handles."""
    specs = [scene_params(*s) for s in SCENES[:4]]
    frames = [[sc.render(f) for f in range(3)] for sc, _ in specs]
    d, c, p = frames[3][0]
    empty = (np.zeros_like(d), c, p)
    batch = Batch([dict(prm, flags=N.VH_FLAG_SYNC | N.VH_FLAG_BATCH_FUSED) for _, prm in specs])
    singles = [Volume(**prm) for _, prm in specs]
    plan = [[0, 1, 2, 3], [0, 2], [1, 3, 0]]
    for k, which in enumerate(plan):
        step = [None] * len(specs)
        for i in which:
            step[i] = empty if (i == 3 and k == 0) else frames[i][k]
        batch.process(step, with_mesh=False)
        status, stats = batch.sync()
        assert status == [0] * len(specs)
        for i in which:
            singles[i].integrate(*step[i])
    for i, v in enumerate(singles):
        assert_same_blocks(batch.scene(i).export_blocks(), v.export_blocks())
        assert batch.scene(i).stats()["blocks_allocated"] == v.stats()["blocks_allocated"]
    batch.close()
