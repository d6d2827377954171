"""Host logic of the batched form's autotuner (clear_gb300/autotune.py), with
the GPU timings replaced by a synthetic cost: the coordinate-descent order
(pool size, then trace block, then shade block, then the sort's radix width),
the configuration it applies, and the JSON cache keyed by the batch's
signature (a second call applies the cached choice without timing)."""
import json

from clear_gb300 import autotune


class FakeBatch:
    """Stands in for batch.BatchRenderer: records what the tuner applies."""

    def __init__(self):
        self.device = "cuda:0"
        self.scenes = [object()] * 3
        self.total_pixels = 4096
        self.offsets = [0, 10, 20, 30]
        self._cfg = {}
        self.radix_bits = 8
        self.rebuilt = []

    def set_config(self, cfg):
        self._cfg = dict(cfg)

    def config(self):
        return dict(self._cfg)

    def rebuild_into_current(self, radix_bits):
        self.rebuilt.append(radix_bits)

    def new_frame(self):
        return "seeds", "pixels"


def _cost(cfg):
    # separable, with its optimum at pool 2 Mi slots, trace block 64, shade block 96
    return ({0: 5.0, 8 << 20: 4.0, 4 << 20: 3.5, 2 << 20: 3.0, 1 << 20: 3.2}[cfg["pool_slots"]]
            + {64: 0.1, 128: 0.3, 256: 0.5}[cfg["trace_block"]]
            + {64: 0.4, 96: 0.2, 128: 0.3}[cfg["shade_block"]])


def _patch(monkeypatch, tmp_path, calls):
    monkeypatch.setenv(autotune.CACHE_ENV, str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "signature", lambda br, depth: f"fake|scenes={len(br.scenes)}|depth={depth}")

    def time_render(br, config, max_depth, seeds, spp=1, graph=True):
        calls.append(("render", dict(config)))
        return _cost(config)

    def time_build(br, radix_bits, reps=3):
        calls.append(("build", radix_bits))
        return {6: 2.0, 7: 1.5, 8: 1.7}[radix_bits]

    monkeypatch.setattr(autotune, "time_render", time_render)
    monkeypatch.setattr(autotune, "time_build", time_build)


def test_coordinate_descent_applies_the_best_configuration(monkeypatch, tmp_path):
    calls = []
    _patch(monkeypatch, tmp_path, calls)
    br = FakeBatch()
    res = autotune.tune(br, max_depth=5)
    assert not res["cached"]
    assert br.config() == {"trace_block": 64, "shade_block": 96, "pool_slots": 2 << 20}
    assert br.radix_bits == 7 and br.rebuilt[-1] == 7 and res["radix_bits"] == 7
    renders = [c for kind, c in calls if kind == "render"]
    n_pool, n_trace = len(autotune.POOL_CANDIDATES), len(autotune.TRACE_BLOCKS)
    assert len(renders) == n_pool + n_trace + len(autotune.SHADE_BLOCKS)
    # pool sizes are tried first at the default blocks, then the trace block at
    # the chosen pool, then the shade block at both choices
    assert all(c["trace_block"] == 128 and c["shade_block"] == 128 for c in renders[:n_pool])
    assert all(c["pool_slots"] == 2 << 20 and c["shade_block"] == 128 for c in renders[n_pool:n_pool + n_trace])
    assert all(c["pool_slots"] == 2 << 20 and c["trace_block"] == 64 for c in renders[n_pool + n_trace:])
    assert [r for kind, r in calls if kind == "build"] == list(autotune.RADIX_BITS)
    assert [t["ms"] for t in res["render_trials"]] == [_cost(c) for c in renders]


def test_cached_choice_is_applied_without_timing(monkeypatch, tmp_path):
    calls = []
    _patch(monkeypatch, tmp_path, calls)
    first = autotune.tune(FakeBatch(), max_depth=5)
    stored = json.loads((tmp_path / "tune.json").read_text())
    assert list(stored) == ["fake|scenes=3|depth=5"]
    calls.clear()
    br = FakeBatch()
    again = autotune.tune(br, max_depth=5)
    assert again["cached"] and calls == []
    assert br.config() == first["config"] and br.radix_bits == first["radix_bits"]
    # another depth is another workload: searched again
    autotune.tune(FakeBatch(), max_depth=8)
    assert any(kind == "render" for kind, _ in calls)
    assert set(json.loads((tmp_path / "tune.json").read_text())) == {"fake|scenes=3|depth=5", "fake|scenes=3|depth=8"}


def test_unreadable_cache_is_ignored(monkeypatch, tmp_path):
    calls = []
    _patch(monkeypatch, tmp_path, calls)
    (tmp_path / "tune.json").write_text("{not json")
    res = autotune.tune(FakeBatch(), max_depth=5)
    assert not res["cached"] and calls
    assert "fake|scenes=3|depth=5" in json.loads((tmp_path / "tune.json").read_text())
