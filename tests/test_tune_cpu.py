"""The batch autotuner's host logic (jpxl_gb300.tune) on the CPU: the sweep
picks the fastest combination, keys bucket workloads, the JSON cache round
trips, and the C ABI exports the tunables."""
import pytest

from jpxl_gb300 import tune


def test_search_picks_the_fastest_combination_and_keeps_every_trial():
    cost = {(2, 2): 9.0, (4, 2): 7.0, (2, 4): 8.0, (4, 4): 5.0, (8, 4): 5.0}
    best, trials = tune.search(lambda l, c: cost.get((l, c), 99.0), lanes=(2, 4, 8),
                               tc_ctas=(2, 4))
    assert (best.lanes, best.tc_ctas_per_sm, best.ms) == (4, 4, 5.0)  # first of equal times
    assert [(t.lanes, t.tc_ctas_per_sm) for t in trials] == [(2, 2), (4, 2), (8, 2),
                                                              (2, 4), (4, 4), (8, 4)]


def test_workload_keys_bucket_sizes():
    a = tune.workload_key("GB300", "bf16x6", 512, 1_000_000_000)
    b = tune.workload_key("GB300", "bf16x6", 600, 1_050_000_000)
    c = tune.workload_key("GB300", "fp32", 512, 1_000_000_000)
    d = tune.workload_key("GB300", "bf16x6", 64, 1_000_000_000)
    assert a == b and a != c and a != d


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("JPXLG_TUNE_CACHE", str(path))
    assert tune.cache_path() == path
    assert tune.tuned_shape("k") is None
    tune.save_cache({"k": {"lanes": 6, "tc_ctas_per_sm": 3, "ms": 1.5}})
    assert tune.tuned_shape("k") == {"lanes": 6, "tc_ctas_per_sm": 3, "ms": 1.5}
    path.write_text("not json")
    assert tune.load_cache() == {}


def test_the_tunable_is_exported():
    lib = pytest.importorskip("jpxl_gb300._lib").load()
    assert hasattr(lib, "jpxlg_tune_set") and hasattr(lib, "jpxlg_tune_get")
