"""The autotuner's host side without a GPU: where its table lives, the table
round trip (and a corrupt or missing table reading as empty), and how a
setting reaches a context's launch parameters."""
import json

from lbvh_gb300 import _lib, autotune


class _FakeCtx:
    def __init__(self):
        self.params = {}

    def set_param(self, param, value):
        self.params[param] = value


def test_cache_path_follows_the_environment(monkeypatch, tmp_path):
    monkeypatch.setenv("LBVH_TUNE_CACHE", str(tmp_path / "t.json"))
    assert autotune.cache_path() == str(tmp_path / "t.json")
    monkeypatch.delenv("LBVH_TUNE_CACHE")
    assert autotune.cache_path().endswith("lbvh_gb300/tuning.json")


def test_table_round_trip_and_bad_tables(tmp_path):
    p = str(tmp_path / "sub" / "tuning.json")
    assert autotune.load_table(p) == {}  # missing
    table = {"k": {"batch_threads": 512, "trace_blocks_per_sm": 8, "trace_refill": 12}}
    autotune.save_table(table, p)  # creates the folder
    assert autotune.load_table(p) == table
    with open(p, "w") as f:
        f.write("{not json")
    assert autotune.load_table(p) == {}
    with open(p, "w") as f:
        json.dump([1, 2], f)  # valid JSON but not a table
    assert autotune.load_table(p) == {}


def test_apply_sets_only_the_given_launch_parameters():
    ctx = _FakeCtx()
    autotune.apply(ctx, {"batch_threads": 1024, "trace_refill": 16, "build_ms": {"256": 1.0}})
    assert ctx.params == {_lib.PARAM_BATCH_THREADS: 1024, _lib.PARAM_TRACE_REFILL: 16}
    autotune.apply(ctx, {"trace_blocks_per_sm": 6})
    assert ctx.params[_lib.PARAM_TRACE_BLOCKS_PER_SM] == 6
    assert set(autotune.BATCH_THREADS) <= {256, 512, 1024}


def test_apply_covers_the_sort_and_traversal_parameters():
    ctx = _FakeCtx()
    autotune.apply(ctx, {"batch_radix_bits": 6, "batch_keys_per_thread": 8, "trace_leaf_batch": 8,
                         "sort_tile_keys": 1024, "bucket_sort_min": 65536, "bounds_blocks_per_sm": 8,
                         "tuned_on": 262267, "build_ms": {"x": 1.0}})
    assert ctx.params == {_lib.PARAM_BATCH_RADIX_BITS: 6, _lib.PARAM_BATCH_KEYS_PER_THREAD: 8,
                          _lib.PARAM_TRACE_LEAF_BATCH: 8, _lib.PARAM_SORT_TILE_KEYS: 1024,
                          _lib.PARAM_BUCKET_SORT_MIN: 65536, _lib.PARAM_BOUNDS_BLOCKS_PER_SM: 8}
    assert set(autotune.BATCH_RADIX_BITS) == {4, 6, 8} and set(autotune.BATCH_KEYS_PER_THREAD) == {4, 8}


def test_build_size_classes_and_candidates(tmp_path):
    assert autotune.size_class(1) == 0 and autotune.size_class(65536) == 16 and autotune.size_class(65535) == 15
    assert autotune.build_key(262267) == "gb300:build:2^18"
    small = autotune.build_candidates(8320)
    assert all(c["bucket_sort_min"] == autotune.BUCKET_SORT_OFF for c in small)  # too small for buckets
    big = autotune.build_candidates(16_000_000)
    assert any(c["bucket_sort_min"] == autotune.BUCKET_SORT_MIN for c in big)
    assert {c["sort_tile_keys"] for c in big} == {0, 1024, 4096}
    # a stored size-class setting reaches a context through apply_build
    p = str(tmp_path / "t.json")
    autotune.save_table({autotune.build_key(300_000): {"sort_tile_keys": 4096, "bounds_blocks_per_sm": 2}}, p)
    ctx = _FakeCtx()
    assert autotune.apply_build(ctx, 262_145, table_path=p) is not None  # same class: 2^18
    assert ctx.params == {_lib.PARAM_SORT_TILE_KEYS: 4096, _lib.PARAM_BOUNDS_BLOCKS_PER_SM: 2}
    assert autotune.apply_build(_FakeCtx(), 600_000, table_path=p) is None
