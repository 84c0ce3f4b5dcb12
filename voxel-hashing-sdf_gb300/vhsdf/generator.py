"""The reference's public classes with their names, arguments and behaviour.

``GpuTsdfGenerator`` mirrors ark::GpuTsdfGenerator (include/tsdf.cuh:548-683,
src/tsdf.cu:1248-1758) and ``HashTable`` mirrors the device hash
vhashing::HashTable (include/vhashing.h:622-826), both forwarding to the
engine's C ABI.  Differences: blocks are 8^3 voxels, the volume stays on the
GPU instead of being streamed through host chunks, allocation follows each
pixel's truncation band, and render() reports that OpenGL is unavailable.
"""
import numpy as np

from . import _native as N
from .engine import Volume


class GpuTsdfGenerator:
    """ark::GpuTsdfGenerator (include/tsdf.cuh:606-607; defaults src/tsdf.cu:1249-1252)."""

    def __init__(self, width, height, fx, fy, cx, cy, max_depth, origin_x=-1.5, origin_y=-1.5,
                 origin_z=0.5, vox_size=0.006, trunc_m=0.03, vox_dim_x=500, vox_dim_y=500,
                 vox_dim_z=500, **engine):
        # origin and dims belong to the reference's dense grid, which its hash
        # path never uses (src/tsdf.cu:621-623 places voxels at index * size).
        self.origin = (origin_x, origin_y, origin_z)
        self.vox_dim = (vox_dim_x, vox_dim_y, vox_dim_z)
        params = dict(width=width, height=height, fx=fx, fy=fy, cx=cx, cy=cy,
                      max_depth=max_depth, voxel_size=vox_size, trunc=trunc_m)
        params.update(engine)
        self.volume = Volume(**params)
        self._vertices = None
        self._faces = None

    def processFrame(self, depth, rgb, c2w):
        """depth: H x W float32 metres; rgb: H x W x 3 uint8 (RGB); c2w: 4x4 row-major."""
        self.volume.process_frame(depth, rgb, c2w)
        self._vertices = self._faces = None

    def SavePLY(self, filename):
        self.volume.save_ply(filename, binary=False)

    def render(self):
        self.volume.render()

    def Shutdown(self):
        self.volume.close()

    def _mesh(self):
        if self._vertices is None:
            v, c, f = self.volume.mesh_indexed()
            self._vertices = (v, c)
            self._faces = f
        return self._vertices, self._faces

    def getVertices(self):
        """(positions in metres [n,3], colours [n,3]) of the full-volume mesh."""
        return self._mesh()[0]

    def getFaces(self):
        return self._mesh()[1]

    def getHashMap(self):
        """The vertex hash of the mesh export (include/tsdf.cuh:637): buckets of
        ((x, y, z, r, g, b), vertex index) keyed by the vertex's voxel cell.
        The reference's insert_vertex works on a copy of the bucket
        (src/tsdf.cu:1935) and leaves its map empty; here it holds every
        merged vertex."""
        (v, c), _ = self._mesh()
        nb = max(1, len(v))
        cells = np.floor(v / self.volume.params.voxel_size).astype(np.int64)
        keys = (cells[:, 0] * 73856093) ^ (cells[:, 1] * 19349669) ^ (cells[:, 2] * 83492791)
        buckets = [[] for _ in range(nb)]
        for i, k in enumerate((keys % nb).tolist()):
            buckets[k].append((tuple(v[i].tolist()) + tuple(c[i].tolist()), i))
        return buckets

    def hash_table(self):
        """The block hash of the volume in the shape of vhashing::HashTable."""
        return HashTable(self.volume)

    def getMarchingCubeParam(self):
        """MarchingCubeParam (include/tsdf.cuh:220-534) as a dict, tables included."""
        p = self.volume.params
        corner = np.zeros((8, 3), np.int32)
        edge = np.zeros(256, np.int32)
        tri = np.zeros((256, 16), np.int32)
        N.lib().vh_mc_tables(corner.ctypes.data, edge.ctypes.data, tri.ctypes.data)
        return {"vox_size": p.voxel_size, "trunc_margin": p.trunc, "max_depth": p.max_depth,
                "min_depth": p.min_depth, "block_size": N.BLOCK_EDGE * p.voxel_size,
                "im_width": p.width, "im_height": p.height, "fx": p.fx, "fy": p.fy,
                "cx": p.cx, "cy": p.cy, "vox_origin": self.origin, "vox_dim": self.vox_dim,
                "total_vox": int(np.prod(self.vox_dim)), "idxMap": corner, "edgeTable": edge,
                "triTable": tri}


class HashTable:
    """vhashing::HashTable over a volume's block hash (include/vhashing.h)."""

    def __init__(self, volume):
        self.volume = volume

    def find(self, keys):
        """Pool index per key or -1 (HashTable::find, include/vhashing.h:128-131)."""
        return self.volume.find_keys(keys)

    def AllocKeys(self, keys):
        """include/vhashing.h:530-603."""
        self.volume.alloc_keys(keys)

    def erase(self, keys):
        """Number of keys erased (include/vhashing.h:244-256)."""
        return self.volume.erase_keys(keys)

    def clearheap(self):
        """include/vhashing.h:80-91."""
        self.volume.clear_block_list()

    @property
    def key_heap(self):
        """Keys of the current block list (include/vhashing.h:55,417-425)."""
        return self.volume.block_list()

    @property
    def heap_counter(self):
        return len(self.volume.block_list())
