"""Host logic of the launch-shape autotuner (no GPU): batch buckets and the
JSON cache round trip."""
import json

from gigalens_gb300.cuda import autotune


def test_batch_buckets_are_powers_of_two():
    assert [autotune._bucket(b) for b in (1, 2, 3, 4, 5, 4096, 4097)] == [1, 2, 4, 4, 8, 4096, 8192]


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "tuning.json"
    monkeypatch.setenv("GIGALENS_GB300_TUNING", str(path))
    autotune.clear_memory_cache()
    try:
        autotune._store("k1", {"choice": {"fused_corr": 2}, "ms": 1.5})
        assert json.loads(path.read_text())["k1"]["choice"] == {"fused_corr": 2}
        autotune.clear_memory_cache()
        assert autotune._load()["k1"]["ms"] == 1.5
    finally:
        autotune.clear_memory_cache()


def test_switch_off(monkeypatch):
    monkeypatch.setenv("GIGALENS_GB300_AUTOTUNE", "0")
    assert not autotune.enabled()
    # with tuning off, ensure_* return at once without touching the plan
    assert autotune.ensure_lstsq(object(), None) is None
    assert autotune.ensure_fused(object(), None) is None
