"""Pythonic handle over the C ABI: one TSDF volume on one GPU.

Arrays may be numpy (host memory) or CUDA torch tensors (device memory of the
volume's GPU); the call passes raw pointers and the memory kind to the
library.  Nothing here computes anything itself.
"""
import ctypes as C

import numpy as np

from . import _native as N


def _is_cuda_tensor(a):
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


class _Arg:
    """Pointer + memory kind of an input array, keeping host copies alive.
    The library reads as many bytes as the volume's parameters say, so the
    size (and for device tensors the GPU) is checked here, before the call."""

    def __init__(self, a, dtype=None):
        if _is_cuda_tensor(a):
            if not a.is_contiguous():
                raise ValueError("device tensors must be contiguous")
            self.keep = a
            self.ptr = a.data_ptr()
            self.mem = N.VH_MEM_DEVICE
            self.dtype = str(a.dtype).replace("torch.", "")
            self.nbytes = a.numel() * a.element_size()
            self.device = a.device.index
        else:
            arr = np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype=dtype))
            self.keep = arr
            self.ptr = arr.ctypes.data
            self.mem = N.VH_MEM_HOST
            self.dtype = str(arr.dtype)
            self.nbytes = arr.nbytes
            self.device = None


def _check_image(arg, params, bytes_per_px, what):
    """`arg` holds exactly one width x height image of `bytes_per_px` bytes
    per pixel, on the volume's GPU if it is a device tensor."""
    want = int(params.width) * int(params.height) * bytes_per_px
    if arg.nbytes != want:
        raise ValueError(f"{what} must hold {params.width}x{params.height} pixels of "
                         f"{bytes_per_px} bytes ({want} bytes), got {arg.nbytes} bytes")
    if arg.mem == N.VH_MEM_DEVICE and arg.device != int(params.device):
        raise ValueError(f"{what} is on cuda:{arg.device}, the volume on cuda:{params.device}")


def _depth_bytes(fmt):
    return 2 if fmt == N.VH_DEPTH_U16_MM else 4


def _depth_arg(depth, params, depth_format=None):
    """A checked depth image and its format."""
    d = _Arg(depth)
    fmt = _depth_fmt(d.dtype, depth_format)
    _check_image(d, params, _depth_bytes(fmt), "depth")
    return d, fmt


def _rgb_arg(rgb, params):
    c = _Arg(rgb, np.uint8)
    if c.mem == N.VH_MEM_DEVICE and c.dtype != "uint8":
        raise TypeError(f"rgb must be uint8, got {c.dtype}")
    _check_image(c, params, 3, "rgb")
    return c


def _depth_fmt(dtype, override=None):
    """uint16 -> scaled integer depth, float32 -> metres.  `override` ("u16" or
    "f32") reinterprets the bytes, e.g. an int16 device tensor holding uint16."""
    if override == "u16" or (override is None and dtype == "uint16"):
        return N.VH_DEPTH_U16_MM
    if override == "f32" or (override is None and dtype == "float32"):
        return N.VH_DEPTH_F32_M
    raise TypeError(f"depth must be uint16 (scaled) or float32 metres, got {dtype}")


class Volume:
    """A voxel-hashed TSDF volume (8^3 blocks) resident on one GPU."""

    def __init__(self, **params):
        self._L = N.lib()
        p = N.VhParams()
        self._L.vh_params_default(C.byref(p))
        for k, v in params.items():
            if not hasattr(p, k):
                raise TypeError(f"unknown parameter {k}")
            setattr(p, k, v)
        self.params = p
        self._pending_meshes = []  # host outputs of vh_process_frame_mesh until sync()
        h = C.c_void_p()
        N.check(self._L.vh_create(C.byref(p), C.byref(h)))
        self._h = h

    # ---- life cycle ----
    def close(self):
        if getattr(self, "_h", None):
            self._L.vh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, status):
        N.check(status, self._h)

    def reset(self):
        self._check(self._L.vh_reset(self._h))

    def sync(self):
        try:
            self._check(self._L.vh_sync(self._h))
        finally:
            self._pending_meshes = []

    def set_stream(self, stream_ptr):
        self._check(self._L.vh_set_stream(self._h, C.c_void_p(stream_ptr)))

    # ---- per-frame path ----
    def _frame_args(self, depth, rgb, c2w, depth_format=None):
        d, fmt = _depth_arg(depth, self.params, depth_format)
        c = _rgb_arg(rgb, self.params)
        if d.mem != c.mem:
            raise ValueError("depth and rgb must both be host or both be device arrays")
        pose = np.ascontiguousarray(np.asarray(c2w, dtype=np.float32).reshape(16))
        return d, fmt, c, pose

    def integrate(self, depth, rgb, c2w, depth_format=None):
        d, fmt, c, pose = self._frame_args(depth, rgb, c2w, depth_format)
        self._check(self._L.vh_integrate(self._h, d.ptr, fmt, c.ptr, pose.ctypes.data, d.mem))

    def process_frame(self, depth, rgb, c2w, depth_format=None):
        d, fmt, c, pose = self._frame_args(depth, rgb, c2w, depth_format)
        self._check(self._L.vh_process_frame(self._h, d.ptr, fmt, c.ptr, pose.ctypes.data, d.mem,
                                             None))

    def process_frame_mesh(self, depth, rgb, c2w, out, count, depth_format=None):
        """process_frame, and the frame's triangles delivered into `out`
        (host float32 array of shape (capacity, 12), the device buffer's
        layout) with the count in count[0] (host int64 array).  Without
        VH_FLAG_SYNC the copy completes by the next sync(); the arrays are
        kept alive until then."""
        d, fmt, c, pose = self._frame_args(depth, rgb, c2w, depth_format)
        if not (isinstance(out, np.ndarray) and out.dtype == np.float32 and out.ndim == 2
                and out.shape[1] == 12 and out.flags.c_contiguous):
            raise ValueError("out must be a C-contiguous float32 array of shape (capacity, 12)")
        if not (isinstance(count, np.ndarray) and count.dtype == np.int64 and count.size >= 1):
            raise ValueError("count must be an int64 array")
        self._pending_meshes.append((out, count))
        self._check(self._L.vh_process_frame_mesh(
            self._h, d.ptr, fmt, c.ptr, pose.ctypes.data, d.mem, out.ctypes.data, out.shape[0],
            count.ctypes.data_as(C.POINTER(C.c_int64))))

    def process_frame_indexed(self, depth, rgb, c2w, verts, faces, counts, depth_format=None):
        """process_frame, and the frame's mesh delivered indexed: vertices
        into `verts` (host float32 array (capacity, 4): x, y, z in voxel
        units and the colour bits), faces into `faces` (host int32 array
        (capacity, 3)), counts[0] = vertices and counts[1] = faces (host
        int64 array).  Without VH_FLAG_SYNC the copy completes by the next
        sync(); the arrays are kept alive until then."""
        d, fmt, c, pose = self._frame_args(depth, rgb, c2w, depth_format)
        if not (isinstance(verts, np.ndarray) and verts.dtype == np.float32 and verts.ndim == 2
                and verts.shape[1] == 4 and verts.flags.c_contiguous):
            raise ValueError("verts must be a C-contiguous float32 array of shape (capacity, 4)")
        if not (isinstance(faces, np.ndarray) and faces.dtype == np.int32 and faces.ndim == 2
                and faces.shape[1] == 3 and faces.flags.c_contiguous):
            raise ValueError("faces must be a C-contiguous int32 array of shape (capacity, 3)")
        if not (isinstance(counts, np.ndarray) and counts.dtype == np.int64 and counts.size >= 2
                and counts.flags.c_contiguous):
            raise ValueError("counts must be an int64 array of two entries")
        self._pending_meshes.append((verts, faces, counts))
        p64 = C.POINTER(C.c_int64)
        self._check(self._L.vh_process_frame_indexed(
            self._h, d.ptr, fmt, c.ptr, pose.ctypes.data, d.mem, verts.ctypes.data, verts.shape[0],
            faces.ctypes.data, faces.shape[0], counts.ctypes.data_as(p64),
            C.cast(counts.ctypes.data + 8, p64)))

    # ---- launch tuning ----
    def tuning(self):
        t = N.VhTuning()
        self._check(self._L.vh_get_tuning(self._h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in N.VhTuning._fields_}

    @staticmethod
    def tuning_variants():
        """(integration shapes, MC shapes): the ranges of integrate_variant
        and mc_variant."""
        a, b = N.I32(), N.I32()
        N.lib().vh_tuning_variants(C.byref(a), C.byref(b))
        return a.value, b.value

    def set_tuning(self, integrate_variant=0, integrate_ctas_per_sm=0, mc_ctas_per_sm=0,
                   mc_variant=0):
        t = N.VhTuning(integrate_variant, integrate_ctas_per_sm, mc_ctas_per_sm, mc_variant)
        self._check(self._L.vh_set_tuning(self._h, C.byref(t)))

    def autotune(self, depth, rgb, c2w, depth_format=None):
        """Times the launch configurations on this frame (scratch volume) and
        applies the fastest; returns it."""
        d, fmt, c, pose = self._frame_args(depth, rgb, c2w, depth_format)
        t = N.VhTuning()
        self._check(self._L.vh_autotune(self._h, d.ptr, fmt, c.ptr, pose.ctypes.data, d.mem,
                                        C.byref(t)))
        return {f: getattr(t, f) for f, _ in N.VhTuning._fields_}

    def extract(self, scope="frame"):
        """Runs marching cubes; returns (device pointer, triangle count)."""
        view = N.VhMeshView()
        sc = N.VH_SCOPE_ALL if scope == "all" else N.VH_SCOPE_FRAME
        self._check(self._L.vh_extract(self._h, sc, C.byref(view)))
        return view.vertices, view.num_triangles

    def mesh(self):
        """Last extraction as (xyz float32 [n,3,3] voxel units, rgb uint8 [n,3,3])."""
        n = C.c_int64()
        self._check(self._L.vh_copy_mesh(self._h, None, None, 0, C.byref(n)))
        xyz = np.empty((n.value, 3, 3), np.float32)
        rgb = np.empty((n.value, 3, 3), np.uint8)
        self._check(self._L.vh_copy_mesh(self._h, xyz.ctypes.data, rgb.ctypes.data, n.value,
                                         C.byref(n)))
        return xyz, rgb

    def stream_out(self, centre, radius):
        """Moves blocks farther than `radius` from `centre` to the host store;
        returns how many moved."""
        c = np.ascontiguousarray(np.asarray(centre, np.float32).reshape(3))
        n = C.c_int64()
        self._check(self._L.vh_stream_out(self._h, c.ctypes.data, float(radius), C.byref(n)))
        return n.value

    def stream_in(self, centre, radius=float("inf")):
        """Moves stored blocks within `radius` of `centre` back; returns how many."""
        c = np.ascontiguousarray(np.asarray(centre, np.float32).reshape(3))
        n = C.c_int64()
        self._check(self._L.vh_stream_in(self._h, c.ctypes.data, float(radius), C.byref(n)))
        return n.value

    def evict_async(self, centre, radius):
        """Moves blocks farther than `radius` from `centre` out of HBM without
        waiting; they reach the host store while later frames run."""
        c = np.ascontiguousarray(np.asarray(centre, np.float32).reshape(3))
        self._check(self._L.vh_evict_async(self._h, c.ctypes.data, float(radius)))

    def compact_table(self):
        self._check(self._L.vh_compact_table(self._h))

    def host_blocks(self):
        return int(self._L.vh_host_blocks(self._h))

    def filter_depth(self, depth, depth_format=None):
        """The VH_FLAG_DEPTH_FILTER pre-filter of one depth image (float metres)."""
        if _is_cuda_tensor(depth):
            raise TypeError("filter_depth takes a host image (the frame path filters device "
                            "images itself with VH_FLAG_DEPTH_FILTER)")
        d, fmt = _depth_arg(depth, self.params, depth_format)
        p = self.params
        out = np.empty((p.height, p.width), np.float32)
        self._check(self._L.vh_filter_depth(self._h, d.ptr, fmt, out.ctypes.data, N.VH_MEM_HOST))
        return out

    def raycast(self, c2w):
        """Ray-cast (depth [H,W] metres (0 = miss), normals [H,W,3] world
        frame, colours [H,W,3]) of the fused surface from pose c2w."""
        p = self.params
        pose = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(16))
        depth = np.empty((p.height, p.width), np.float32)
        normal = np.empty((p.height, p.width, 3), np.float32)
        rgb = np.empty((p.height, p.width, 3), np.uint8)
        self._check(self._L.vh_raycast(self._h, pose.ctypes.data, depth.ctypes.data,
                                       normal.ctypes.data, rgb.ctypes.data, N.VH_MEM_HOST))
        return depth, normal, rgb

    def mesh_indexed(self):
        """Full-volume mesh with vertices merged on the GPU: (vertices [n,3]
        metres float32, colours [n,3] uint8, faces [m,3] int32)."""
        nv, nf = C.c_int64(), C.c_int64()
        self._check(self._L.vh_mesh_indexed(self._h, None, None, 0, None, 0, C.byref(nv),
                                            C.byref(nf)))
        v = np.empty((nv.value, 3), np.float32)
        c = np.empty((nv.value, 3), np.uint8)
        f = np.empty((nf.value, 3), np.int32)
        self._check(self._L.vh_mesh_indexed(self._h, v.ctypes.data, c.ctypes.data, nv.value,
                                            f.ctypes.data, nf.value, C.byref(nv), C.byref(nf)))
        return v, c, f

    def save_ply(self, path, binary=False):
        self._check(self._L.vh_save_ply(self._h, str(path).encode(), int(binary)))

    def render(self):
        self._check(self._L.vh_render(self._h))

    # ---- hash surface ----
    def _keys(self, keys):
        if _is_cuda_tensor(keys):
            a = _Arg(keys)
            if a.dtype != "int32" or keys.numel() % 3:
                raise TypeError("device keys must be an int32 tensor of (x, y, z) triples")
            if a.device != int(self.params.device):
                raise ValueError(f"keys are on cuda:{a.device}, the volume on "
                                 f"cuda:{self.params.device}")
            return a, keys.numel() // 3
        k = np.ascontiguousarray(np.asarray(keys, dtype=np.int32).reshape(-1, 3))
        return _Arg(k), k.shape[0]

    def alloc_keys(self, keys):
        a, n = self._keys(keys)
        self._check(self._L.vh_alloc_keys(self._h, a.ptr, n, a.mem))

    def find_keys(self, keys):
        a, n = self._keys(keys)
        if a.mem == N.VH_MEM_DEVICE:
            import torch
            out = torch.empty(n, dtype=torch.int32, device=keys.device)
            self._check(self._L.vh_find_keys(self._h, a.ptr, n, out.data_ptr(), a.mem))
            return out
        out = np.empty(n, np.int32)
        self._check(self._L.vh_find_keys(self._h, a.ptr, n, out.ctypes.data, a.mem))
        return out

    def erase_keys(self, keys):
        a, n = self._keys(keys)
        cnt = C.c_int64()
        self._check(self._L.vh_erase_keys(self._h, a.ptr, n, C.byref(cnt), a.mem))
        return cnt.value

    def clear_block_list(self):
        self._check(self._L.vh_clear_block_list(self._h))

    def block_list(self):
        n = C.c_int64()
        self._check(self._L.vh_block_list(self._h, None, 0, C.byref(n)))
        out = np.empty((n.value, 3), np.int32)
        self._check(self._L.vh_block_list(self._h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def device_table(self):
        """The vh_device_table of this volume (device addresses of the hash
        and the block pool) for kernels compiled against
        include/vhashing_device.cuh."""
        t = N.VhDeviceTable()
        self._check(self._L.vh_get_device_table(self._h, C.byref(t)))
        return t

    # ---- gradients and pose refinement ----
    def sdf_sample(self, xyz):
        """Trilinear sdf (units of T), gradient (per metre) and validity at
        world points; numpy in, numpy out (torch CUDA tensors: device path)."""
        if _is_cuda_tensor(xyz):
            import torch
            a = _Arg(xyz)
            if a.dtype != "float32" or xyz.numel() % 3:
                raise TypeError("device points must be a float32 tensor of (x, y, z) triples")
            if a.device != int(self.params.device):
                raise ValueError(f"points are on cuda:{a.device}, the volume on "
                                 f"cuda:{self.params.device}")
            n = xyz.numel() // 3
            phi = torch.empty(n, dtype=torch.float32, device=xyz.device)
            grad = torch.empty((n, 3), dtype=torch.float32, device=xyz.device)
            valid = torch.empty(n, dtype=torch.uint8, device=xyz.device)
            self._check(self._L.vh_sdf_sample(self._h, xyz.data_ptr(), n, phi.data_ptr(),
                                              grad.data_ptr(), valid.data_ptr(), N.VH_MEM_DEVICE))
            return phi, grad, valid.bool()
        pts = np.ascontiguousarray(np.asarray(xyz, np.float32).reshape(-1, 3))
        n = pts.shape[0]
        phi = np.empty(n, np.float32)
        grad = np.empty((n, 3), np.float32)
        valid = np.empty(n, np.uint8)
        self._check(self._L.vh_sdf_sample(self._h, pts.ctypes.data, n, phi.ctypes.data,
                                          grad.ctypes.data, valid.ctypes.data, N.VH_MEM_HOST))
        return phi, grad, valid.astype(bool)

    def pose_normal_equations(self, depth, c2w, stride=1, method="adjoint", depth_format=None):
        d, fmt = _depth_arg(depth, self.params, depth_format)
        pose = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(16))
        out = np.empty(29, np.float64)
        m = N.VH_REFINE_FD if method == "fd" else N.VH_REFINE_ADJOINT
        self._check(self._L.vh_pose_normal_equations(self._h, d.ptr, fmt, d.mem,
                                                     pose.ctypes.data, stride, m,
                                                     out.ctypes.data))
        return out

    def pose_refine(self, depth, c2w, iterations=20, stride=1, method="adjoint",
                    depth_format=None):
        """Gauss-Newton refinement of a camera pose against the volume;
        returns (refined 4x4 c2w, stats dict)."""
        d, fmt = _depth_arg(depth, self.params, depth_format)
        pose = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(16))
        out = np.empty(16, np.float32)
        st = N.VhRefineStats()
        m = N.VH_REFINE_FD if method == "fd" else N.VH_REFINE_ADJOINT
        self._check(self._L.vh_pose_refine(self._h, d.ptr, fmt, d.mem,
                                           pose.ctypes.data, iterations, stride, m,
                                           out.ctypes.data, C.byref(st)))
        return out.reshape(4, 4), {f: getattr(st, f) for f, _ in N.VhRefineStats._fields_}

    def pose_refine_batch(self, depths, c2ws, iterations=20, stride=1, depth_format=None):
        """Adjoint refinement of n poses together, pose i against depths[i]
        (all host arrays or all CUDA tensors, one dtype; depth_format as in
        process_frame); returns (n x 4 x 4 refined c2w, list of n stats)."""
        args = [_Arg(d) for d in depths]
        n = len(args)
        if n == 0 or any(a.mem != args[0].mem or a.dtype != args[0].dtype for a in args):
            raise ValueError("depths must be one memory kind and dtype, at least one image")
        fmt = _depth_fmt(args[0].dtype, depth_format)
        for a in args:
            _check_image(a, self.params, _depth_bytes(fmt), "depth")
        tab = (C.c_void_p * n)(*[a.ptr for a in args])
        poses = np.ascontiguousarray(np.asarray(c2ws, np.float32).reshape(n, 16))
        out = np.empty((n, 16), np.float32)
        st = (N.VhRefineStats * n)()
        self._check(self._L.vh_pose_refine_batch(self._h, C.cast(tab, C.c_void_p), fmt,
                                                 args[0].mem, n,
                                                 poses.ctypes.data, iterations, stride,
                                                 out.ctypes.data, st))
        stats = [{f: getattr(x, f) for f, _ in N.VhRefineStats._fields_} for x in st]
        return out.reshape(n, 4, 4), stats

    def integrate_vjp(self, depth, c2w, grad_sdf):
        """dL/ddepth (H x W) and dL/dxi (6) of the last integration, given
        dL/dsdf per voxel of the block list (n_blocks x 512, host arrays)."""
        d, fmt = _depth_arg(depth, self.params)
        pose = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(16))
        g = np.ascontiguousarray(grad_sdf, np.float32)
        nb = C.c_int64()
        self._check(self._L.vh_block_list(self._h, None, 0, C.byref(nb)))
        if g.size != nb.value * N.BLOCK_VOXELS:
            raise ValueError(f"grad_sdf must hold {nb.value} x {N.BLOCK_VOXELS} values (one per "
                             f"voxel of the block list), got {g.size}")
        gd = np.empty((self.params.height, self.params.width), np.float32)
        gp = np.empty(6, np.float32)
        self._check(self._L.vh_integrate_vjp(self._h, d.ptr, fmt,
                                             pose.ctypes.data, g.ctypes.data, gd.ctypes.data,
                                             gp.ctypes.data, N.VH_MEM_HOST))
        return gd, gp

    # ---- volume I/O ----
    def export_blocks(self):
        n = C.c_int64()
        self._check(self._L.vh_export_blocks(self._h, None, None, None, None, 0, C.byref(n)))
        m = n.value
        xyz = np.empty((m, 3), np.int32)
        sdf = np.empty((m, N.BLOCK_VOXELS), np.float32)
        w = np.empty((m, N.BLOCK_VOXELS), np.float32)
        rgb = np.empty((m, N.BLOCK_VOXELS, 3), np.uint8)
        self._check(self._L.vh_export_blocks(self._h, xyz.ctypes.data, sdf.ctypes.data,
                                             w.ctypes.data, rgb.ctypes.data, m, C.byref(n)))
        return {"xyz": xyz, "sdf": sdf, "weight": w, "rgb": rgb}

    def import_blocks(self, xyz, sdf, weight, rgb):
        xyz = np.ascontiguousarray(xyz, np.int32).reshape(-1, 3)
        sdf = np.ascontiguousarray(sdf, np.float32)
        weight = np.ascontiguousarray(weight, np.float32)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        n = xyz.shape[0]
        for name, a, per in (("sdf", sdf, 1), ("weight", weight, 1), ("rgb", rgb, 3)):
            if a.size != n * N.BLOCK_VOXELS * per:
                raise ValueError(f"{name} must hold {n} x {N.BLOCK_VOXELS}"
                                 f"{' x 3' if per == 3 else ''} values, got {a.size}")
        self._check(self._L.vh_import_blocks(self._h, xyz.ctypes.data, sdf.ctypes.data,
                                             weight.ctypes.data, rgb.ctypes.data, xyz.shape[0]))

    def save(self, path):
        self._check(self._L.vh_save(self._h, str(path).encode()))

    def load(self, path):
        self._check(self._L.vh_load(self._h, str(path).encode()))

    def stats(self):
        s = N.VhStats()
        self._check(self._L.vh_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in N.VhStats._fields_}


def block_hash_ref(x, y, z):
    """The reference's BlockHasher value (include/tsdf.cuh:144-156)."""
    return int(N.lib().vh_block_hash_ref(int(x), int(y), int(z)))


def decode_depth_png(data):
    """A grayscale PNG depth image (bytes) as a (height, width) uint16 array,
    decoded by the library (vh_decode_depth_png): the millimetre frames the
    reference reads with cv::imread (src/SaveFrame.cpp:174-180), ready for
    Volume.integrate as VH_DEPTH_U16_MM."""
    buf = np.frombuffer(bytes(data), np.uint8)
    L = N.lib()
    w, h = C.c_int32(), C.c_int32()
    N.check(L.vh_decode_depth_png(buf.ctypes.data, buf.size, None, 0, C.byref(w), C.byref(h)))
    out = np.empty((h.value, w.value), np.uint16)
    N.check(L.vh_decode_depth_png(buf.ctypes.data, buf.size, out.ctypes.data, out.size,
                                  C.byref(w), C.byref(h)))
    return out


def decode_colour_png(data):
    """A PNG colour image (bytes) as a (height, width, 3) uint8 RGB array,
    decoded by the library (vh_decode_colour_png): what the reference gets
    from cv::imread(path, IMREAD_COLOR) and its BGR-to-RGB swap
    (src/SaveFrame.cpp:164, src/main.cpp:273)."""
    buf = np.frombuffer(bytes(data), np.uint8)
    L = N.lib()
    w, h = C.c_int32(), C.c_int32()
    N.check(L.vh_decode_colour_png(buf.ctypes.data, buf.size, None, 0, C.byref(w), C.byref(h)))
    out = np.empty((h.value, w.value, 3), np.uint8)
    N.check(L.vh_decode_colour_png(buf.ctypes.data, buf.size, out.ctypes.data, out.size,
                                   C.byref(w), C.byref(h)))
    return out


def decode_colour_jpeg(data):
    """A JPEG colour image (bytes) as a (height, width, 3) uint8 RGB array,
    decoded by the library (vh_decode_colour_jpeg): the <i>.jpg colour
    frames the reference reads with cv::imread (src/SaveFrame.cpp:164)."""
    buf = np.frombuffer(bytes(data), np.uint8)
    L = N.lib()
    w, h = C.c_int32(), C.c_int32()
    N.check(L.vh_decode_colour_jpeg(buf.ctypes.data, buf.size, None, 0, C.byref(w), C.byref(h)))
    out = np.empty((h.value, w.value, 3), np.uint8)
    N.check(L.vh_decode_colour_jpeg(buf.ctypes.data, buf.size, out.ctypes.data, out.size,
                                    C.byref(w), C.byref(h)))
    return out


def resize_colour(rgb, width, height):
    """An RGB uint8 image (h, w, 3) resized bilinearly to (height, width, 3)
    by the library (vh_resize_colour), as the reference scales its colour
    frames to the depth grid with cv::resize (src/SaveFrame.cpp:164-171)."""
    src = np.ascontiguousarray(rgb, np.uint8)
    if src.ndim != 3 or src.shape[2] != 3:
        raise ValueError(f"rgb must have shape (h, w, 3), got {src.shape}")
    out = np.empty((int(height), int(width), 3), np.uint8)
    N.check(N.lib().vh_resize_colour(src.ctypes.data, src.shape[1], src.shape[0],
                                     out.ctypes.data, out.shape[1], out.shape[0]))
    return out
