"""Volume snapshots, PLY export and the reference-named front ends."""
import numpy as np
import pytest

from helpers import assert_same_blocks, oracle_for, small_scene, volume_for
from vhsdf import GpuTsdfGenerator, HashTable, VhError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(gpu):
    return small_scene()


def test_snapshot_round_trip(scene, tmp_path):
    vol = volume_for(scene)
    for f in range(4):
        vol.integrate(*scene.render(f))
    path = tmp_path / "vol.vhs"
    vol.save(path)
    other = volume_for(scene)
    other.load(path)
    assert_same_blocks(other.export_blocks(), vol.export_blocks())
    # integration continues identically after a reload
    vol.integrate(*scene.render(4))
    other.integrate(*scene.render(4))
    assert_same_blocks(other.export_blocks(), vol.export_blocks())


def read_ply(path):
    with open(path, "rb") as f:
        header = []
        while True:
            line = f.readline().decode().strip()
            header.append(line)
            if line == "end_header":
                break
        nv = int([h for h in header if h.startswith("element vertex")][0].split()[-1])
        nf = int([h for h in header if h.startswith("element face")][0].split()[-1])
        binary = any("binary_little_endian" in h for h in header)
        if binary:
            vdt = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("r", "u1"), ("g", "u1"),
                            ("b", "u1")])
            v = np.frombuffer(f.read(nv * vdt.itemsize), vdt)
            fdt = np.dtype([("n", "u1"), ("i", "<i4", 3)])
            fc = np.frombuffer(f.read(nf * fdt.itemsize), fdt)
            return np.stack([v["x"], v["y"], v["z"]], -1), fc["i"], fc["n"]
        rows = [f.readline().split() for _ in range(nv)]
        v = np.array([[float(r[0]), float(r[1]), float(r[2])] for r in rows])
        fr = [f.readline().split() for _ in range(nf)]
        return v, np.array([[int(r[1]), int(r[2]), int(r[3])] for r in fr]), \
            np.array([int(r[0]) for r in fr])


@pytest.mark.parametrize("binary", [False, True])
def test_ply_export(scene, tmp_path, binary):
    vol = volume_for(scene)
    for f in range(3):
        vol.integrate(*scene.render(f))
    path = tmp_path / "mesh.ply"
    vol.save_ply(path, binary=binary)
    v, faces, nper = read_ply(path)
    vol.extract("all")
    xyz, _ = vol.mesh()
    assert len(faces) == len(xyz) and np.all(nper == 3)
    uniq = np.unique(xyz.reshape(-1, 3), axis=0)
    assert len(v) == len(uniq)
    assert faces.min() >= 0 and faces.max() < len(v)
    vs = vol.params.voxel_size
    got = np.sort(v[faces].reshape(-1, 3), axis=0)
    want = np.sort((xyz * np.float32(vs)).reshape(-1, 3).astype(np.float64), axis=0)
    assert np.allclose(got, want, atol=1e-5 if not binary else 0)


def test_gpu_tsdf_generator_front_end(scene, tmp_path):
    """ark::GpuTsdfGenerator surface: float metre depth, RGB, row-major c2w."""
    gen = GpuTsdfGenerator(scene.width, scene.height, scene.fx, scene.fy, scene.cx, scene.cy,
                           4.5, vox_size=0.02, trunc_m=0.08, table_log2=18,
                           pool_blocks=1 << 16, max_frame_blocks=1 << 16)
    orc = oracle_for(gen.volume, 32)
    for f in range(3):
        d, c, p = scene.render(f)
        dm = d.astype(np.float32) * np.float32(0.001)
        gen.processFrame(dm, c, p.reshape(-1))
        orc.integrate(dm, c, p)
    assert_same_blocks(gen.volume.export_blocks(), orc.export())
    gen.SavePLY(str(tmp_path / "g.ply"))
    verts, cols = gen.getVertices()
    faces = gen.getFaces()
    assert verts.shape[1] == 3 and cols.shape == verts.shape and faces.max() < len(verts)
    mc = gen.getMarchingCubeParam()
    assert abs(mc["block_size"] - 0.16) < 1e-7
    assert mc["edgeTable"][1] == 0x109 and list(mc["triTable"][1][:3]) == [0, 8, 3]
    assert mc["idxMap"].tolist()[1] == [0, 1, 0]  # the reference's corner order
    vmap = gen.getHashMap()
    assert sorted(i for bucket in vmap for _, i in bucket) == list(range(len(verts)))
    with pytest.raises(VhError):
        gen.render()
    table = gen.hash_table()
    assert isinstance(table, HashTable)
    keys = gen.volume.export_blocks()["xyz"][:5]
    assert np.all(table.find(keys) >= 0)
    table.clearheap()
    assert table.heap_counter == 0
    table.AllocKeys(np.array([[500, 500, 500]], np.int32))
    assert table.heap_counter == 1 and table.erase(np.array([[500, 500, 500]], np.int32)) == 1
    gen.Shutdown()


def merged_mesh_reference(xyz, rgb, voxel):
    """The vertex merge of tsdf2mesh (src/tsdf.cu:1777,1810-1821) over the
    triangles sorted by (vertex coordinates, colours): exact-position merge,
    numbering and colour by first occurrence.  numpy restatement."""
    n = len(xyz)
    p = xyz.reshape(n, 9).astype(np.float32)
    p = np.where(p == 0, np.float32(0), p)  # -0 == +0
    c = (rgb.reshape(n, 3, 3).astype(np.uint32) * np.array([1, 256, 65536], np.uint32)).sum(-1)
    keys = [c[:, 2], c[:, 1], c[:, 0]] + [p[:, k] for k in range(8, -1, -1)]
    order = np.lexsort(keys)
    occ = p[order].reshape(-1, 3)
    occ_rgb = rgb[order].reshape(-1, 3)
    view = np.ascontiguousarray(occ).view(np.dtype((np.void, 12))).ravel()
    _, first, inverse = np.unique(view, return_index=True, return_inverse=True)
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(len(first))
    faces = rank[inverse.ravel()].reshape(-1, 3).astype(np.int32)
    fo = np.sort(first)
    verts = occ[fo] * np.float32(voxel)
    return verts.astype(np.float32), occ_rgb[fo], faces


def test_gpu_vertex_merge_matches_reference_rule(scene, tmp_path):
    vol = volume_for(scene)
    for f in range(5):
        vol.integrate(*scene.render(f))
    v, c, faces = vol.mesh_indexed()
    vol.extract("all")
    xyz, rgb = vol.mesh()
    rv, rc, rf = merged_mesh_reference(xyz, rgb, vol.params.voxel_size)
    assert len(v) == len(rv) and len(faces) == len(rf) > 0
    assert np.array_equal(v.view(np.uint32), rv.view(np.uint32))
    assert np.array_equal(c, rc)
    assert np.array_equal(faces, rf)
    # the binary PLY carries exactly these arrays
    path = tmp_path / "m.ply"
    vol.save_ply(path, binary=True)
    pv, pf, nper = read_ply(path)
    assert np.array_equal(pv.astype(np.float32).view(np.uint32), v.view(np.uint32))
    assert np.array_equal(pf, faces) and np.all(nper == 3)
    # and repeated calls give the same bytes (no dependence on GPU scheduling)
    path2 = tmp_path / "m2.ply"
    vol.save_ply(path2, binary=True)
    assert path.read_bytes() == path2.read_bytes()


def test_bad_snapshot_leaves_the_volume_unchanged(scene, tmp_path):
    """A snapshot that the import would reject (a fractional weight, more
    blocks than the pool holds) is refused before the volume is cleared."""
    vol = volume_for(scene)
    for f in range(3):
        vol.integrate(*scene.render(f))
    good = tmp_path / "good.vhs"
    vol.save(good)
    n = len(vol.export_blocks()["xyz"])
    raw = bytearray(good.read_bytes())
    header = 8 + 4 + 4 + 4 + 4 + 8
    w_off = header + 12 * n + 2048 * n  # first weight of the first block
    raw[w_off:w_off + 4] = np.float32(0.5).tobytes()
    bad = tmp_path / "bad_weight.vhs"
    bad.write_bytes(bytes(raw))

    other = volume_for(scene)
    other.integrate(*scene.render(5))
    before = other.export_blocks()
    with pytest.raises(VhError):
        other.load(bad)
    assert_same_blocks(other.export_blocks(), before)
    small = volume_for(scene, pool_blocks=max(n // 2, 4))
    small.alloc_keys(np.array([[0, 0, 0], [1, 0, 0]], np.int32))
    before = small.export_blocks()
    assert len(before["xyz"]) == 2
    with pytest.raises(VhError):
        small.load(good)
    assert_same_blocks(small.export_blocks(), before)
