"""The C ABI library on the CPU: it loads, exports every symbol include/crt.h
declares, refuses to run without an sm_103a GPU (no host fallback), and the
drop-in adapter compiles and links against the reference's own bvh.hpp."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "crt.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(crt_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from realtimeraytracing_gb300 import build, crt
    build.build()
    return crt.lib()


def test_every_declared_symbol_is_exported(lib):
    from realtimeraytracing_gb300 import crt
    decl = _declared()
    assert len(decl) >= 20
    for name in decl:
        assert hasattr(lib, name), name
    assert sorted(crt.EXPORTS) == decl


def test_abi_version(lib):
    assert lib.crt_abi_version() == 1


def test_no_gpu_means_an_error_not_a_fallback(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from realtimeraytracing_gb300 import crt
    with pytest.raises(crt.CrtError) as e:
        crt.Context()
    assert e.value.status == 6  # CRT_ERR_UNSUPPORTED


def test_invalid_config_rejected(lib):
    from realtimeraytracing_gb300 import crt
    with pytest.raises(crt.CrtError) as e:
        crt.Context(ploc_radius=0)
    assert e.value.status == 1
    with pytest.raises(crt.CrtError):
        crt.Context(sort_digit_bits=5)


def test_struct_sizes_match_reference_records(tmp_path):
    code = r'''
#include <stdio.h>
#include <stddef.h>
#include "crt.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(crt_triangle), sizeof(crt_mesh_model),
         sizeof(crt_bvh_node), sizeof(crt_ray), sizeof(crt_hit), offsetof(crt_bvh_node, mx),
         offsetof(crt_bvh_node, tri), offsetof(crt_bvh_node, right), offsetof(crt_triangle, model_id),
         sizeof(crt_material), sizeof(crt_shading), offsetof(crt_shading, bvh_depth));
  return 0;
}'''
    src = tmp_path / "sizes.c"
    src.write_text(code)
    exe = str(tmp_path / "sizes")
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    # TriangleGPU 64, MeshModelGPU 68, BVH_NodeGPU 48 (max @16, tri @32, right @40), MaterialGPU 16
    assert [int(x) for x in out] == [64, 68, 48, 32, 16, 16, 32, 40, 48, 16, 40, 32]
    from realtimeraytracing_gb300 import crt
    assert C.sizeof(crt.Shading) == 40 and crt.Shading.bvh_depth.offset == 32


def _reference_dir():
    from oracle import oracle as O
    return O.REFERENCE_DIR


@pytest.mark.skipif(not os.path.isdir(os.path.join(_reference_dir(), "srcCommon")),
                    reason="reference checkout not present")
def test_adapter_compiles_and_links_against_reference_header(lib, tmp_path):
    gxx = shutil.which("g++")
    tmp = str(tmp_path)
    inc = ["-I", os.path.join(ROOT, "oracle", "glm_shim"), "-I",
           os.path.join(_reference_dir(), "srcCommon", "scene", "geometry"),
           "-I", os.path.join(ROOT, "include")]
    obj = os.path.join(tmp, "bvh_cuda.o")
    subprocess.run([gxx, "-std=gnu++20", "-O2", "-c", os.path.join(ROOT, "adapter", "bvh_cuda.cpp"), *inc, "-o", obj],
                   check=True)
    main = os.path.join(tmp, "main.cpp")
    with open(main, "w") as f:
        f.write('#include "bvh.hpp"\nint main(){ std::vector<cr::TriangleGPU> t(4); '
                'std::vector<cr::MeshModelGPU> m(cr::Mesh::MAX_NB_MESHES); cr::BVH b(4, t, m); return 0; }\n')
    libdir = os.path.join(ROOT, "realtimeraytracing_gb300")
    subprocess.run([gxx, "-std=gnu++20", main, obj, *inc, "-L", libdir, "-lcrt", f"-Wl,-rpath,{libdir}",
                    "-o", os.path.join(tmp, "main")], check=True)


LAYOUT_PROBE = r"""
#include <cstddef>
#include <cstdio>
#include <typeinfo>
#include "bvh.hpp"
#define OFF(T, m) std::printf(#T "." #m " %zu\n", offsetof(cr::T, m))
int main() {
    std::printf("TriangleGPU %zu MeshModelGPU %zu AABB_GPU %zu BVH_NodeGPU %zu\n", sizeof(cr::TriangleGPU),
                sizeof(cr::MeshModelGPU), sizeof(cr::AABB_GPU), sizeof(cr::BVH_NodeGPU));
    OFF(TriangleGPU, _P1); OFF(TriangleGPU, _P2); OFF(TriangleGPU, _ModelId); OFF(MeshModelGPU, _MaterialId);
    OFF(AABB_GPU, _Max); OFF(BVH_NodeGPU, _TriangleId); OFF(BVH_NodeGPU, _LeftChild); OFF(BVH_NodeGPU, _RightChild);
    std::printf("%s\n%s\n%s\n%s\n%s\n%s\n%s\n%s\n", typeid(decltype(cr::BVH_Params::_Clusters)).name(),
                typeid(decltype(cr::BVH_Params::_IsLeaf)).name(), typeid(decltype(cr::BVH_Params::_Parent)).name(),
                typeid(decltype(cr::BVH_Params::_LeftChild)).name(), typeid(decltype(cr::BVH_Params::_RightChild)).name(),
                typeid(decltype(cr::BVH_Params::_TriangleIndices)).name(), typeid(decltype(cr::BVH_Params::_UnsortedTriangles)).name(),
                typeid(decltype(cr::BVH::_InternalStruct)).name());
    std::printf("%u %zu\n", static_cast<unsigned>(cr::Triangle::MAX_NB_TRIANGLES), sizeof(cr::BVH_Params::_NbTriangles));
    return 0;
}
"""


@pytest.mark.skipif(not os.path.isdir(os.path.join(_reference_dir(), "srcCommon")),
                    reason="reference checkout not present")
def test_adapter_stand_in_header_matches_the_reference_header(tmp_path):
    """tests/adapter_iface/bvh.hpp (used to run the adapter where the
    reference checkout is absent) declares the reference header's records
    with the same sizes and member offsets, and BVH_Params members of the
    same types."""
    gxx = shutil.which("g++")
    src = os.path.join(str(tmp_path), "probe.cpp")
    with open(src, "w") as f:
        f.write(LAYOUT_PROBE)
    outs = []
    for hdr in (os.path.join(_reference_dir(), "srcCommon", "scene", "geometry"), os.path.join(ROOT, "tests", "adapter_iface")):
        exe = os.path.join(str(tmp_path), "probe")
        subprocess.run([gxx, "-std=gnu++20", "-w", src, "-I", hdr, "-I", os.path.join(ROOT, "oracle", "glm_shim"),
                        "-o", exe], check=True)
        outs.append(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)
    assert outs[0] == outs[1], outs
