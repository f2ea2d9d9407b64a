"""The C++ drop-in header against the reference's own lbvh.h (where the
reference's files are present: $LBVH_REF_DIR, or the copy staged in
baseline/_ref), as a maintainer switching lbvh::builder<float> to
lbvh::gpu::builder<float> would: compiled on every machine, and on a GPU run
side by side with the reference builder and traverser in one process."""
import os
import subprocess
import tempfile

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.ref_dir()
HAVE_REF = os.path.exists(os.path.join(REF, "lbvh.h"))

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

# The reference's builder and traverser next to the drop-ins on the same
# input, in one process: a seeded triangle soup (and a second, larger one),
# pinhole rays through the scene; node arrays compared byte for byte, hits
# field for field (primitive, distance bits, uv bits). lbvh_test.cpp:154-175
# and 327-347 drive the reference the same way (builder, then one traverser
# call per ray).
RUN_SRC = r"""
#include <lbvh.h>
#include "lbvh_gpu.hpp"
#include <cstdio>
#include <cstring>
#include <random>

using namespace lbvh;

static int compare(size_t n, unsigned seed) {
  std::mt19937 rng(seed);
  std::uniform_real_distribution<float> c(-1.0f, 1.0f);
  std::normal_distribution<float> d(0.0f, 0.05f);
  std::vector<triangle<float>> tris;
  for (size_t i = 0; i < n; i++) {
    const float x = c(rng), y = c(rng), z = c(rng);
    tris.emplace_back(vec3<float>{x + d(rng), y + d(rng), z + d(rng)},
                      vec3<float>{x + d(rng), y + d(rng), z + d(rng)},
                      vec3<float>{x + d(rng), y + d(rng), z + d(rng)});
  }
  builder<float> cpu_builder;
  bvh<float> want = cpu_builder(tris.data(), tris.size(), triangle_aabb_converter<float>());
  gpu::builder<float> gpu_builder;
  bvh<float> got = gpu_builder(tris.data(), tris.size(), triangle_aabb_converter<float>());
  if (got.size() != want.size() || std::memcmp(&got[0], &want[0], want.size() * sizeof(node<float>)) != 0) {
    std::printf("nodes differ (n=%zu)\n", n);
    return 1;
  }
  const int w = 96, h = 64;
  std::vector<ray<float>> rays;
  for (int j = 0; j < h; j++)
    for (int i = 0; i < w; i++) {
      const float u = (i + 0.5f) / w * 2.0f - 1.0f, v = (j + 0.5f) / h * 2.0f - 1.0f;
      rays.push_back(ray<float>{{0, 0, 3}, {u * 0.6f, v * 0.4f, -1.0f}});
    }
  traverser<float, triangle<float>, triangle_intersection<float>> cpu_trav(want, tris.data());
  gpu::traverser<float, triangle<float>, triangle_intersection<float>> gpu_trav(got, tris.data());
  std::vector<gpu::traverser<float, triangle<float>, triangle_intersection<float>>::intersection> ghits(rays.size());
  gpu_trav.trace(rays.data(), rays.size(), ghits.data());
  size_t bad = 0, hits = 0;
  for (size_t k = 0; k < rays.size(); k++) {
    const auto a = cpu_trav(rays[k], triangle_intersector<float>());
    const auto& b = ghits[k];
    const auto one = gpu_trav(rays[k], triangle_intersector<float>());
    bool same = a.primitive == b.primitive && one.primitive == a.primitive;
    if (same && a.primitive != std::numeric_limits<uint32_t>::max()) {
      hits++;
      same = std::memcmp(&a.info.distance, &b.info.distance, 4) == 0 &&
             std::memcmp(&a.info.uv.x, &b.info.uv.x, 4) == 0 && std::memcmp(&a.info.uv.y, &b.info.uv.y, 4) == 0 &&
             std::memcmp(&a.info.distance, &one.info.distance, 4) == 0;
    }
    bad += !same;
  }
  std::printf("n=%zu nodes=%zu rays=%zu hits=%zu mismatches=%zu\n", n, want.size(), rays.size(), hits, bad);
  return bad ? 1 : 0;
}

int main() {
  try {
    int rc = compare(968, 1);
    rc |= compare(20000, 2);
    return rc;
  } catch (const gpu::error& e) {
    std::printf("error %d: %s\n", e.status(), e.what());
    return 2;
  }
}
"""


def _compile(d, src_text, lib):
    src = os.path.join(d, "t.cpp")
    with open(src, "w") as f:
        f.write(src_text)
    exe = os.path.join(d, "t")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-Wno-class-memaccess",
                        "-I", REF, "-I", os.path.join(ROOT, "include"), src, "-o", exe, lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-pthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.mark.skipif(not HAVE_REF, reason="reference header not staged on this machine")
def test_drop_in_header_compiles_against_reference(lib_built):
    with tempfile.TemporaryDirectory() as d:
        _compile(d, SRC, lib_built)
        _compile(d, RUN_SRC, lib_built)


@pytest.mark.gpu
@pytest.mark.skipif(not HAVE_REF, reason="reference header not staged on this machine")
def test_drop_in_matches_reference_in_one_process(lib_built):
    """gpu::builder's bvh<float> bytes equal lbvh::builder<float>'s, and
    gpu::traverser's hits (batch and per-ray) equal lbvh::traverser's."""
    with tempfile.TemporaryDirectory() as d:
        exe = _compile(d, RUN_SRC, lib_built)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        assert r.stdout.count("mismatches=0") == 2, r.stdout
