"""The batched autotuner's JSON cache (simall_autotune_cache_lookup / _store,
host only): round trips, replacement, several keys, a missing file, damaged
lines and invalid keys."""
import json

from simall_gb300.batch import autotune_cache_lookup, autotune_cache_store


def test_round_trip_and_replace(tmp_path):
    p = str(tmp_path / "sub" / "dir" / "autotune.json")  # parent directories are created
    assert autotune_cache_lookup(p, "k1") is None
    assert autotune_cache_store(p, "k1", (1024, 1, 2, 0, 0, 0), 12.5) == 0
    assert autotune_cache_store(p, "k2|GB300|sm152", (512, 2, 1, 32768, 16, 2), 3.25) == 0
    assert autotune_cache_lookup(p, "k1") == (1024, 1, 2, 0, 0, 0)
    assert autotune_cache_lookup(p, "k2|GB300|sm152") == (512, 2, 1, 32768, 16, 2)
    assert autotune_cache_store(p, "k1", (256, 4, 4, 16384, 8, 6), 1.0) == 0
    assert autotune_cache_lookup(p, "k1") == (256, 4, 4, 16384, 8, 6)
    doc = json.load(open(p))  # the file is valid JSON
    assert doc["k1"] == {"block_threads": 256, "ctas_per_sm": 4, "rows_per_pass": 4, "cluster_rows": 16384,
                         "cluster_ctas": 8, "clusters": 6, "ms": 1.0}
    assert set(doc) == {"k1", "k2|GB300|sm152"}


def test_damaged_lines_are_dropped(tmp_path):
    p = tmp_path / "autotune.json"
    p.write_text('{\n "good": {"block_threads": 512, "ctas_per_sm": 2, "rows_per_pass": 1, "cluster_rows": 0, '
                 '"cluster_ctas": 0, "clusters": 0, "ms": 2.000},\n "bad": {"block_threads": oops},\n'
                 ' "old": {"block_threads": 512, "ctas_per_sm": 2, "rows_per_pass": 1, "ms": 2.000},\n garbage\n')
    assert autotune_cache_lookup(str(p), "good") == (512, 2, 1, 0, 0, 0)
    assert autotune_cache_lookup(str(p), "old") is None  # an entry of an earlier format
    assert autotune_cache_lookup(str(p), "bad") is None
    assert autotune_cache_store(str(p), "new", (1024, 1, 1, 0, 0, 0)) == 0
    doc = json.load(open(p))
    assert set(doc) == {"good", "new"}


def test_invalid_arguments(tmp_path):
    p = str(tmp_path / "a.json")
    assert autotune_cache_store(p, 'bad"key', (1, 1, 1, 0, 0, 0)) == 1  # SIMALL_ERR_INVALID_ARGUMENT
    assert autotune_cache_store(p, "", (1, 1, 1, 0, 0, 0)) == 1
    assert autotune_cache_store("", "k", (1, 1, 1, 0, 0, 0)) == 1
    assert autotune_cache_lookup(p, "k") is None
