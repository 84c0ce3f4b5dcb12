"""GPU path vs the CPU oracle, through the C ABI.

Bar: allocated block set and triangle count bit-exact; with the fp32
oracle every stored value is bit-exact too; against the FP64 oracle sdf is
within 1e-5 (absolute, sdf is in [-1, 1]), weight exact, colour within one
level, vertices within 1e-4 voxel plus one fp32 ulp of the coordinate.
"""
import numpy as np
import pytest
import torch

from helpers import (assert_same_blocks, key_set, oracle_for, small_scene, sort_rows,
                     sorted_blocks, tri_rows, volume_for)
from vhsdf import Volume

pytestmark = pytest.mark.gpu

SDF_TOL = 1e-5
VERTEX_TOL = 1e-4


@pytest.fixture(scope="module")
def scene(gpu):
    return small_scene()


def test_allocation_set_is_bit_exact(scene):
    vol = volume_for(scene)
    orc = oracle_for(vol)
    seen = set()
    for f in range(0, 20, 3):
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
        want = key_set(orc.band_blocks(d, p))
        got = vol.block_list()
        assert len(got) == len(key_set(got)), "frame block list has duplicates"
        assert key_set(got) == want, f"frame {f}"
        seen |= want
        st = vol.stats()
        assert st["frame_blocks"] == len(want)
    e = vol.export_blocks()
    assert key_set(e["xyz"]) == seen
    assert vol.stats()["blocks_allocated"] == len(seen)


def test_integration_is_bit_exact_with_fp32_oracle(scene):
    vol = volume_for(scene)
    orc = oracle_for(vol, 32)
    for f in range(8):
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
        orc.integrate(d, c, p)
        assert vol.stats()["voxels_updated"] == orc.counts()["voxels_updated"]
    assert_same_blocks(vol.export_blocks(), orc.export())


def test_integration_within_tolerance_of_fp64_oracle(scene):
    vol = volume_for(scene)
    orc = oracle_for(vol, 64)
    for f in range(8):
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
        orc.integrate(d, c, p)
    g = sorted_blocks(vol.export_blocks())
    o = sorted_blocks(orc.export(fp64=True))
    assert np.array_equal(g["xyz"], o["xyz"])
    assert np.array_equal(g["weight"].astype(np.float64), o["weight64"])
    err = np.abs(g["sdf"].astype(np.float64) - o["sdf64"])
    assert err.max() <= SDF_TOL * np.maximum(1.0, np.abs(o["sdf64"])).max()
    assert np.abs(g["rgb"].astype(int) - o["rgb"].astype(int)).max() <= 1


@pytest.mark.parametrize("scope", ["all", "frame"])
def test_marching_cubes_bit_exact(scene, scope):
    vol = volume_for(scene)
    orc = oracle_for(vol, 32)
    for f in range(6):
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
        orc.integrate(d, c, p)
    vol.extract(scope)
    gx, gc = vol.mesh()
    m = orc.marching_cubes(scope)
    assert len(gx) == len(m["xyz"]) > 100
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))


def test_marching_cubes_vs_fp64_on_identical_volume(scene):
    """FP64 oracle MC of the GPU's own TSDF: same triangle count, vertices
    within tolerance."""
    vol = volume_for(scene)
    for f in range(6):
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
    e = vol.export_blocks()
    orc = oracle_for(vol, 64)
    orc.import_blocks(e["xyz"], e["sdf"], e["weight"], e["rgb"])
    vol.extract("all")
    gx, gc = vol.mesh()
    m = orc.marching_cubes("all")
    assert len(gx) == len(m["xyz"])
    order_g = np.lexsort(tri_rows(gx, gc).T[::-1])
    order_o = np.lexsort(tri_rows(m["xyz"], m["rgb"]).T[::-1])
    a = gx[order_g].astype(np.float64)
    b = m["xyz64"][order_o]
    ulp = np.spacing(np.abs(b).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(a - b) <= VERTEX_TOL + ulp)


def test_gpu_mc_on_oracle_volume(scene):
    """Import the oracle's volume into the engine: MC agrees bit for bit."""
    orc = None
    vol = volume_for(scene)
    orc = oracle_for(vol, 32)
    for f in range(4):
        d, c, p = scene.render(f)
        orc.integrate(d, c, p)
    o = orc.export()
    vol.import_blocks(o["xyz"], o["sdf"], o["weight"], o["rgb"])
    assert_same_blocks(vol.export_blocks(), o)
    vol.extract("all")
    gx, gc = vol.mesh()
    m = orc.marching_cubes("all")
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))


def test_input_formats_and_memory_kinds_agree(scene):
    """u16 vs f32 depth, host vs device buffers, graph vs direct launches."""
    from vhsdf import _native as N
    exports = []
    for mode in ("u16_host", "f32_host", "u16_device", "f32_device_nograph"):
        flags = N.VH_FLAG_SYNC | (N.VH_FLAG_NO_GRAPH if "nograph" in mode else 0)
        vol = volume_for(scene, flags=flags)
        for f in range(5):
            d, c, p = scene.render(f)
            if mode.startswith("f32"):
                d = d.astype(np.float32) * np.float32(0.001)
            if "device" in mode:
                dt = torch.from_numpy(d.astype(np.int16) if d.dtype == np.uint16 else d).cuda()
                ct = torch.from_numpy(c).cuda()
                vol.process_frame(dt, ct, p, depth_format="u16" if d.dtype == np.uint16 else "f32")
            else:
                vol.process_frame(d, c, p)
        exports.append(sorted_blocks(vol.export_blocks()))
        vol.close()
    for e in exports[1:]:
        for k in ("xyz", "sdf", "weight", "rgb"):
            assert np.array_equal(e[k], exports[0][k]), k


def test_ragged_image_size_and_odd_intrinsics(gpu):
    scene = small_scene(w=97, h=61)
    vol = volume_for(scene, voxel=0.03, trunc=0.1)
    orc = oracle_for(vol, 32)
    for f in range(0, 20, 4):
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
        orc.integrate(d, c, p)
        assert key_set(vol.block_list()) == key_set(orc.band_blocks(d, p))
    assert_same_blocks(vol.export_blocks(), orc.export())
    vol.extract("all")
    gx, gc = vol.mesh()
    m = orc.marching_cubes("all")
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))


def test_invalid_depth_values_are_skipped_like_the_oracle(scene):
    vol = volume_for(scene)
    orc = oracle_for(vol, 32)
    d, c, p = scene.render(2)
    df = d.astype(np.float32) * np.float32(0.001)
    rng = np.random.default_rng(7)
    idx = rng.integers(0, df.size, 4000)
    df.reshape(-1)[idx[:1000]] = np.nan
    df.reshape(-1)[idx[1000:2000]] = np.inf
    df.reshape(-1)[idx[2000:3000]] = -1.0
    df.reshape(-1)[idx[3000:]] = 9.0  # beyond max_depth
    vol.integrate(df, c, p)
    orc.integrate(df, c, p)
    assert_same_blocks(vol.export_blocks(), orc.export())


def test_frame_scope_mc_after_list_change_without_integration(scene):
    """Import / alloc_keys change the block list without integrating; the
    per-frame extraction must then rebuild its neighbour table."""
    vol = volume_for(scene)
    orc = oracle_for(vol, 32)
    for f in range(4):
        orc.integrate(*scene.render(f))
    o = orc.export()
    vol.import_blocks(o["xyz"], o["sdf"], o["weight"], o["rgb"])  # list = imported keys
    lst = vol.block_list()
    orc.set_frame(lst)
    vol.extract("frame")
    gx, gc = vol.mesh()
    m = orc.marching_cubes("frame")
    assert len(gx) == len(m["xyz"]) > 100
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))
    # erase half the listed blocks: their cubes and neighbours disappear
    vol.erase_keys(lst[::2])
    keep = lst[1::2]
    orc2 = oracle_for(vol, 32)
    e = vol.export_blocks()
    orc2.import_blocks(e["xyz"], e["sdf"], e["weight"], e["rgb"])
    orc2.set_frame(keep)
    vol.extract("frame")
    gx, gc = vol.mesh()
    m = orc2.marching_cubes("frame")
    assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))


def test_every_launch_configuration_is_bit_exact(scene):
    """The tuner only changes speed: each configuration (every integration
    shape and every MC shape, some with reduced grids) reproduces the oracle."""
    orc = None
    results = []
    ni, nm = Volume.tuning_variants()
    assert ni >= 6 and nm >= 3
    configs = [(iv, 0, 0, iv % nm) for iv in range(ni)] + [(0, 2, 3, 1), (1, 1, 1, 0), (3, 1, 2, 2)]
    for cfg in configs:
        vol = volume_for(scene)
        vol.set_tuning(*cfg)
        if orc is None:
            orc = oracle_for(vol, 32)
            for f in range(4):
                orc.integrate(*scene.render(f))
        for f in range(4):
            vol.process_frame(*scene.render(f))
        assert_same_blocks(vol.export_blocks(), orc.export())
        vol.extract("all")
        results.append(sort_rows(tri_rows(*vol.mesh())))
        vol.close()
    m = orc.marching_cubes("all")
    want = sort_rows(tri_rows(m["xyz"], m["rgb"]))
    for r in results:
        assert np.array_equal(r, want)


def test_autotune_picks_a_valid_configuration(scene, tmp_path, monkeypatch):
    monkeypatch.setenv("VHSDF_TUNING_CACHE", str(tmp_path / "tune.txt"))
    vol = volume_for(scene)
    d, c, p = scene.render(0)
    t = vol.autotune(d, c, p)
    ni, nm = Volume.tuning_variants()
    assert 0 <= t["integrate_variant"] < ni and 0 <= t["mc_variant"] < nm
    assert t["integrate_ctas_per_sm"] >= 1 and t["mc_ctas_per_sm"] >= 1
    assert vol.stats()["blocks_allocated"] == 0  # the handle's volume is untouched
    assert vol.tuning() == t
    assert (tmp_path / "tune.txt").read_text().strip()
    vol2 = volume_for(scene)
    assert vol2.autotune(d, c, p) == t  # served from the cache


@pytest.mark.parametrize("mc_variant", [0, 1, 2])
def test_frame_meshes_of_each_mc_variant(scene, mc_variant):
    """Per-frame marching cubes of each kernel variant equals the oracle's."""
    vol = volume_for(scene)
    vol.set_tuning(0, 0, 0, mc_variant)
    orc = oracle_for(vol, 32)
    for f in range(4):
        d, c, p = scene.render(f)
        vol.process_frame(d, c, p)
        orc.integrate(d, c, p)
        gx, gc = vol.mesh()
        m = orc.marching_cubes("frame")
        assert len(gx) > 0
        assert np.array_equal(sort_rows(tri_rows(gx, gc)), sort_rows(tri_rows(m["xyz"], m["rgb"])))


def test_mc_on_dense_sign_changes(scene):
    """Random signs cut about half of every block's edges (up to five
    triangles per cube, every candidate round full): the mesh still equals
    the oracle's."""
    rng = np.random.default_rng(9)
    n = 40
    xyz = np.stack([rng.integers(-3, 3, n), rng.integers(-3, 3, n), rng.integers(-3, 3, n)], -1)
    xyz = np.unique(xyz, axis=0).astype(np.int32)
    m = len(xyz)
    sdf = rng.uniform(-1, 1, (m, 512)).astype(np.float32)
    w = np.ones((m, 512), np.float32)
    rgb = rng.integers(0, 256, (m, 512, 3)).astype(np.uint8)
    want = None
    for variant in range(Volume.tuning_variants()[1]):
        vol = volume_for(scene)
        vol.set_tuning(0, 0, 0, variant)
        vol.import_blocks(xyz, sdf, w, rgb)
        vol.extract("all")
        got = sort_rows(tri_rows(*vol.mesh()))
        if want is None:
            orc = oracle_for(vol, 32)
            orc.import_blocks(xyz, sdf, w, rgb)
            mm = orc.marching_cubes("all")
            want = sort_rows(tri_rows(mm["xyz"], mm["rgb"]))
        assert len(got) > 5000
        assert np.array_equal(got, want)
        vol.close()


def test_colour_average_at_every_weight_range(scene):
    """Voxels imported with weights at the edges of the colour average's
    paths (first observation; umulhi up to w_old 2047; corrected reciprocal
    up to 65536; the fp32 formula beyond) and random colours: one integrated
    frame equals the fp32 oracle bit for bit."""
    vol = volume_for(scene)
    seed_orc = oracle_for(vol, 32)
    seed_orc.integrate(*scene.render(0))
    e = seed_orc.export()
    rng = np.random.default_rng(11)
    levels = np.array([0, 1, 2, 3, 254, 255, 256, 1023, 2046, 2047, 2048, 2049, 65535, 65536,
                       65537, 1e6, 2 ** 24], np.float32)
    w = levels[rng.integers(0, len(levels), e["weight"].shape)]
    rgb = rng.integers(0, 256, e["rgb"].shape).astype(np.uint8)
    vol.import_blocks(e["xyz"], e["sdf"], w, rgb)
    orc = oracle_for(vol, 32)
    orc.import_blocks(e["xyz"], e["sdf"], w, rgb)
    for f in (1, 2):
        d, c, p = scene.render(f)
        vol.integrate(d, c, p)
        orc.integrate(d, c, p)
    g = vol.export_blocks()
    assert_same_blocks(g, orc.export())
    # every weight range was updated (w_old = 2^24 stays: 2^24 + 1 rounds back)
    pos = {k: i for i, k in enumerate(map(tuple, g["xyz"].tolist()))}
    idx = np.array([pos[k] for k in map(tuple, e["xyz"].tolist())])
    changed = g["weight"][idx] != w
    for lv in levels[:-1]:
        assert np.any(changed & (w == lv)), lv
    vol.close()
