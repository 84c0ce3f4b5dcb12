"""Builds the native libraries in-tree with nvcc / g++ (no cmake).

    lib/libvhsdf.so        the engine: CUDA kernels for sm_103a + C ABI
    lib/libvhsdf_checked.so  the same with the per-frame kernels compiled with
                           VH_CHECKED (index checks that record an error and
                           skip the access; selected by VHSDF_CHECKED=1)
    lib/libvhsynth.so      synthetic RGB-D scene generator (OpenMP)
    ../oracle/lib/libvh_oracle.so   CPU oracle used by tests and the benchmark

Objects are rebuilt only when a source is newer than the library.
    python build_native.py [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(PKG, "lib", "obj")
ORACLE = os.path.join(REPO, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
               "-I" + os.path.join(REPO, "include")] + ARCH
# -fmad=false: decisions and stored values are single IEEE roundings so the
# CPU oracle reproduces them bit for bit.
KERNEL_FLAGS = ["-fmad=false", "--prec-div=true", "--prec-sqrt=true"]

# host code whose floating-point results must not depend on the machine:
# no contraction of a * b + c into a fused multiply-add (gcc contracts by
# default on aarch64, not on x86-64)
HOST_EXACT = ["-Xcompiler", "-ffp-contract=off"]
ENGINE_SOURCES = [
    ("vh_kernels.cu", KERNEL_FLAGS),
    ("vh_api.cpp", []),
    ("vh_mesh.cpp", []),
    ("vh_noalloc.cu", []),
    ("vh_adjoint.cu", []),
    ("vh_batch.cpp", []),
    ("vh_meshindex.cu", []),
    ("vh_raycast.cu", []),
    ("vh_stream.cu", []),
    ("vh_png.cpp", []),
    ("vh_frames.cpp", HOST_EXACT),
    ("vh_jpeg.cpp", HOST_EXACT),
]
ENGINE_HEADERS = ["vh_common.cuh", "vh_device.cuh", "vh_mc_tables.h", "vh_mesh.h", "vh_internal.h"]

ENGINE_LIB = os.path.join(LIB, "libvhsdf.so")
CHECKED_LIB = os.path.join(LIB, "libvhsdf_checked.so")
CHECKED_SOURCE = "vh_kernels.cu"  # where the VH_CHECK sites are
SYNTH_LIB = os.path.join(LIB, "libvhsynth.so")
ORACLE_LIB = os.path.join(ORACLE, "lib", "libvh_oracle.so")


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build vhsdf")
    return exe


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_engine(force=False):
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in ENGINE_HEADERS] + [
        os.path.join(REPO, "include", "vhsdf.h")]
    srcs = [os.path.join(CSRC, s) for s, _ in ENGINE_SOURCES]
    deps = srcs + headers + [__file__]
    if not force and not _newer(ENGINE_LIB, deps) and not _newer(CHECKED_LIB, deps):
        return ENGINE_LIB
    jobs = []
    objs = []
    checked_objs = []
    for name, extra in ENGINE_SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ, name + ".o")
        objs.append(obj)
        jobs.append([nvcc()] + NVCC_COMMON + extra + ["-c", src, "-o", obj])
        if name == CHECKED_SOURCE:
            cobj = os.path.join(OBJ, name + ".checked.o")
            checked_objs.append(cobj)
            jobs.append([nvcc()] + NVCC_COMMON + extra + ["-DVH_CHECKED", "-c", src, "-o", cobj])
        else:
            checked_objs.append(obj)
    with cf.ThreadPoolExecutor(len(jobs)) as ex:
        list(ex.map(_run, jobs))
    with cf.ThreadPoolExecutor(2) as ex:
        list(ex.map(_run, [[nvcc()] + ARCH + ["-shared", "-o", ENGINE_LIB] + objs,
                           [nvcc()] + ARCH + ["-shared", "-o", CHECKED_LIB] + checked_objs]))
    return ENGINE_LIB


def build_synth(force=False):
    os.makedirs(LIB, exist_ok=True)
    src = os.path.join(PKG, "synth", "vh_synth.cpp")
    if force or _newer(SYNTH_LIB, [src, __file__]):
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", SYNTH_LIB])
    return SYNTH_LIB


def build_oracle(force=False):
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = os.path.join(ORACLE, "vh_oracle.cpp")
    if force or _newer(ORACLE_LIB, [src, __file__]):
        # -ffp-contract=off: no fused multiply-add, the operation order of the
        # source is the rounding order (matches the GPU's -fmad=false).
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              src, "-o", ORACLE_LIB])
    return ORACLE_LIB


def build_all(force=False):
    with cf.ThreadPoolExecutor(3) as ex:
        futs = [ex.submit(build_engine, force), ex.submit(build_synth, force),
                ex.submit(build_oracle, force)]
        return [f.result() for f in futs]


if __name__ == "__main__":
    for p in build_all(force="--force" in sys.argv):
        print(p)
