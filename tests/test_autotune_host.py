"""Host logic of the launch-shape autotuner (no GPU): batch buckets, the
JSON cache round trip, and the least-squares search order with the timing
and the plan calls faked."""
import json

import torch

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


def test_lstsq_search_times_basis_shapes_then_gram_kernels(tmp_path, monkeypatch):
    """ensure_lstsq times the six basis shapes, then the two Gram kernels on
    the fastest shape; it applies and caches the overall fastest, counts one
    timed plan shape, and a second plan of the same shape takes the cache."""
    monkeypatch.setenv("GIGALENS_GB300_TUNING", str(tmp_path / "tuning.json"))
    monkeypatch.setenv("GIGALENS_GB300_AUTOTUNE", "1")
    autotune.clear_memory_cache()
    applied = []
    cost = {(1, -1): 9.0, (1, 16): 8.0, (1, 20): 5.0, (2, -1): 7.0, (2, 16): 6.0, (2, 20): 5.5}
    state = {}

    def fake_set(plan, lsq_ctas_per_sm=0, lsq_col_block=0, fused_corr=0, lsq_gram=0):
        if lsq_ctas_per_sm:
            state["shape"] = (lsq_ctas_per_sm, lsq_col_block)
        state["gram"] = lsq_gram or state.get("gram", 2)
        applied.append(dict(lsq_ctas_per_sm=lsq_ctas_per_sm, lsq_col_block=lsq_col_block, lsq_gram=lsq_gram))

    def fake_time(bench, reps, warmup=2):
        return cost[state["shape"]] - (1.0 if state["gram"] == 1 else 0.0)   # the tensor-core Gram faster here

    monkeypatch.setattr(autotune, "set_tuning", fake_set)
    monkeypatch.setattr(autotune, "_time_ms", fake_time)
    monkeypatch.setattr(autotune, "plan_key", lambda plan, kind, bs: "lstsq|fake")

    class FakePlan:
        pass

    try:
        t0, c0 = autotune.stats["timed"], autotune.stats["cached"]
        x = torch.zeros(4, 3)
        choice = autotune.ensure_lstsq(FakePlan(), x)
        assert choice == dict(lsq_ctas_per_sm=1, lsq_col_block=20, lsq_gram=1)
        # six basis shapes with the plan's Gram kernel, then the two kernels on (1, 20)
        shapes = [(a["lsq_ctas_per_sm"], a["lsq_col_block"]) for a in applied[:6]]
        assert sorted(shapes) == sorted(cost)
        assert [a["lsq_gram"] for a in applied[7:9]] == [2, 1]
        assert applied[-1] == dict(lsq_ctas_per_sm=1, lsq_col_block=20, lsq_gram=1)
        assert autotune.stats["timed"] == t0 + 1
        autotune.clear_memory_cache()
        applied.clear()
        assert autotune.ensure_lstsq(FakePlan(), x) == choice
        assert autotune.stats["cached"] == c0 + 1 and applied == [choice]
    finally:
        autotune.clear_memory_cache()
