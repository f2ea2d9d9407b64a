"""The C++ drop-in header compiled against the reference's own lbvh.h (where
the reference tree is present), as a maintainer switching
lbvh::builder<float> to lbvh::gpu::builder<float> would."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("LBVH_REF_DIR", "/root/reference")

SRC = r"""
#include <lbvh.h>
#include "lbvh_gpu.hpp"
#include <cstdio>

int main() {
  using namespace lbvh;
  std::vector<triangle<float>> tris;
  for (int i = 0; i < 16; i++)
    tris.emplace_back(vec3<float>{float(i), 0, 0}, vec3<float>{float(i) + 1, 0, 0}, vec3<float>{float(i), 1, 0});
  try {
    gpu::builder<float> builder;
    bvh<float> b = builder(tris.data(), tris.size(), triangle_aabb_converter<float>());
    gpu::traverser<float, triangle<float>, triangle_intersection<float>> trav(b, tris.data());
    auto hit = trav(ray<float>{{0.5f, 0.25f, 1}, {0, 0, -1}}, triangle_intersector<float>());
    auto boxes_bvh = builder(tris.data(), tris.size(), [](const triangle<float>& t) {
      return triangle_aabb_converter<float>()(t);
    });
    std::printf("%zu %u %zu\n", b.size(), hit.primitive, boxes_bvh.size());
  } catch (const gpu::error& e) {
    std::printf("error %d: %s\n", e.status(), e.what());
    return 2;
  }
  return 0;
}
"""


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "lbvh.h")), reason="reference header not on this machine")
def test_drop_in_header_compiles_against_reference(lib_built):
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        with open(src, "w") as f:
            f.write(SRC)
        r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Wno-class-memaccess", "-I", REF,
                            "-I", os.path.join(ROOT, "include"), src, "-o", os.path.join(d, "t"), lib_built,
                            "-pthread"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
