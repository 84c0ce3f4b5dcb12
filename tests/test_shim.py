"""The header-only ark::GpuTsdfGenerator front end (include/ark_tsdf.h)
compiles with the reference's call pattern and links against the engine."""
import os
import subprocess

import pytest

from conftest import PKG, REPO, cuda_available

# The calls PointCloudGenerator makes (src/PointCloudGenerator.cpp:43-45,
# 118-136): construct from camera/voxel settings, processFrame with float
# metres, RGB bytes and a row-major cam2base, then SavePLY.
PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "ark_tsdf.h"
#include "vhashing_table.h"

int main(int argc, char **argv) {
  const int w = 64, h = 48;
  ark::GpuTsdfGenerator *gen =
      new ark::GpuTsdfGenerator(w, h, 50.f, 50.f, 31.5f, 23.5f, 4.0f, 0.5f, 0.0f, -0.5f,
                                0.01f, 0.04f, 200, 200, 200);
  if (gen->last_status() != VH_OK) {
    std::printf("status %d\n", (int)gen->last_status());
    delete gen;
    return 0;
  }
  std::vector<float> depth(w * h, 1.0f);
  std::vector<unsigned char> rgb(w * h * 3, 128);
  float cam2base[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  for (int f = 0; f < 3; ++f)
    if (gen->processFrame(depth.data(), rgb.data(), cam2base) != VH_OK) return 2;
  if (argc > 1) gen->SavePLY(argv[1]);
  size_t mapped = 0;
  for (const auto &bucket : *gen->getHashMap()) mapped += bucket.size();
  const ark::MarchingCubeParam *mc = gen->getMarchingCubeParam();
  std::printf("ok %zu %zu %zu %d %d %g\n", gen->getVertices()->size(), gen->getFaces()->size(),
              mapped, mc->edgeTable[1], mc->triTable[1][2], mc->block_size);
  // the block hash in vhashing::HashTable's shape
  vhashing::BlockHashTable table(gen->handle());
  const std::vector<vhashing::BlockKey> heap = table.key_heap();
  int found = 0;
  for (int id : table.find(heap)) found += id >= 0;
  table.clearheap();
  const long long cleared = table.heap_counter();
  table.AllocKeys({{500, 500, 500}});
  const long long allocated = table.heap_counter();
  const long long erased = table.erase({{500, 500, 500}});
  std::printf("hash %zu %d %lld %lld %lld %d\n", heap.size(), found, cleared, allocated, erased,
              (int)table.last_status());
  gen->Shutdown();
  delete gen;
  return 0;
}
"""


def build_program(tmp_path):
    src = tmp_path / "uses_shim.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "uses_shim"
    lib = os.path.join(PKG, "lib")
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-I", os.path.join(REPO, "include"),
                    "-L", lib, "-lvhsdf", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    return exe


def test_shim_compiles_and_links(tmp_path):
    exe = build_program(tmp_path)
    if not cuda_available():
        out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
        assert out.returncode == 0
        assert out.stdout.strip() == "status 11"  # VH_ERR_NO_DEVICE, no exception, no exit()


@pytest.mark.gpu
def test_shim_fuses_a_plane(tmp_path, gpu):
    exe = build_program(tmp_path)
    ply = tmp_path / "plane.ply"
    out = subprocess.run([str(exe), str(ply)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    first, second = out.stdout.strip().splitlines()
    _, nv, nf, nm, e1, t12, bs = first.split()
    assert int(nv) > 100 and int(nf) > 100
    assert int(nm) == int(nv)  # every merged vertex in the vertex hash
    assert int(e1) == 0x109 and int(t12) == 3 and abs(float(bs) - 0.08) < 1e-6  # tables, 8 voxels
    _, heap, found, cleared, allocated, erased, status = second.split()
    assert int(heap) > 0 and int(found) == int(heap)
    assert (int(cleared), int(allocated), int(erased), int(status)) == (0, 1, 1, 0)
    header = ply.read_bytes().split(b"end_header")[0].decode()
    assert f"element face {nf}" in header


def test_headers_compile_without_warnings(tmp_path):
    """vhsdf.h is plain C (C99); the C++ front ends compile warning-free
    under strict flags, so they can be dropped into a caller's build."""
    c_src = tmp_path / "c_api.c"
    c_src.write_text('#include "vhsdf.h"\nint main(void) { vh_params p; '
                     'return vh_params_default(&p) == VH_OK ? 0 : 1; }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Wpedantic", "-Werror", "-c",
                    str(c_src), "-I", os.path.join(REPO, "include"), "-o",
                    str(tmp_path / "c_api.o")], check=True)
    cpp_src = tmp_path / "uses_shim.cpp"
    cpp_src.write_text(PROGRAM)
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Wpedantic", "-Wshadow",
                    "-Wconversion", "-Werror", "-c", str(cpp_src), "-I",
                    os.path.join(REPO, "include"), "-o", str(tmp_path / "uses_shim.o")],
                   check=True)
