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
