"""The C ABI library without a GPU: it loads, exports every function the
public header declares, and the header compiles as C and C++."""
import ctypes
import os
import subprocess
import tempfile

import pytest

from lbvh_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(lib_built):
    L = ctypes.CDLL(lib_built)
    declared = _lib.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing
    # the Python binding covers the whole header
    assert set(declared) == set(_lib.SIGNATURES)


def test_host_only_entry_points(lib_built):
    L = _lib.lib()
    assert L.lbvh_version() == 100
    assert L.lbvh_status_string(0).decode() == "ok"
    assert L.lbvh_status_string(3).decode() == "device wait timed out"
    # null-argument checks run before any CUDA call
    assert L.lbvh_ctx_create(0, None, None) == _lib.LBVH_ERR_INVALID_ARG
    assert L.lbvh_ctx_destroy(None) == _lib.LBVH_ERR_INVALID_ARG
    assert L.lbvh_bvh_info(None, None, None, None) == _lib.LBVH_ERR_INVALID_ARG


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_header_compiles(lib_built, lang):
    src = r"""
#include "lbvh_gb300.h"
int main(void) {
  lbvh_ctx* ctx = 0;
  int st = lbvh_ctx_create(0, 0, &ctx);
  return st == LBVH_OK ? 0 : (int)sizeof(lbvh_node) + (int)sizeof(lbvh_hit);
}
"""
    with tempfile.TemporaryDirectory() as d:
        ext = "c" if lang == "c" else "cpp"
        path = os.path.join(d, "t." + ext)
        with open(path, "w") as f:
            f.write(src)
        cc = "gcc" if lang == "c" else "g++"
        exe = os.path.join(d, "t")
        r = subprocess.run([cc, "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), path, "-o", exe,
                            lib_built], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """With the CUDA library absent the package raises instead of computing
    anything on the CPU."""
    import lbvh_gb300 as lb

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "liblbvh_gb300.so"))
    with pytest.raises(ImportError, match="no CPU fallback"):
        _lib.lib()
    with pytest.raises(ImportError):
        lb.Context(0, 0)
