"""The autotuner's cache logic (hcorepp_gb300/autotune.py), without a GPU: stack-width classes, keys,
fallback to the defaults, a store / lookup round trip, and coordinate descent over a fake timer."""
import json
import sys
import types

import numpy as np

from hcorepp_gb300 import autotune as A


def test_classes_and_keys():
    assert [A.stack_class(x) for x in (0, 16, 17, 45.5, 128, 129, 5000)] == [16, 16, 32, 64, 128, 256, 1024]
    assert A.cache_key(512, 45.5, "plain_fp64") == "nb512-k64-plain_fp64"
    comp = np.array([[False, True], [True, False]])
    assert A.mean_stack_width(np.array([[512, 10], [20, 512]]), np.array([[0, 30], [40, 0]]), comp) == 50.0


def test_lookup_falls_back_and_round_trips(tmp_path):
    path = str(tmp_path / "cache.json")
    assert A.lookup("nb512-k64-plain_fp64", A.load(path)) == A.DEFAULT
    cfg = {"groups": 16, "wy_min": 96, "oz_min": 4096, "graph": 1, "precond": 32}
    A.store("nb512-k64-plain_fp64", cfg, {"groups=16": 800.0}, path)
    A.store("nb1024-k128-mixed_ff48", A.DEFAULT, {}, path)
    cache = A.load(path)
    assert A.lookup("nb512-k64-plain_fp64", cache) == cfg
    assert A.lookup("nb512-k64-mixed_ff48", cache) == A.DEFAULT
    assert set(json.load(open(path))) == {"nb512-k64-plain_fp64", "nb1024-k128-mixed_ff48"}


def test_committed_cache_is_well_formed():
    for key, ent in A.load().items():
        assert key.startswith("nb") and "-k" in key
        assert set(ent["config"]) <= set(A.DEFAULT)  # knobs added later fall back to their defaults
        for knob, v in ent["config"].items():
            assert v in A.CANDIDATES[knob]


def test_coordinate_descent_picks_the_fastest(monkeypatch):
    # a fake context and timer: the cost is a known function of the knobs
    applied = []

    class Ctx:
        def set_concurrency(self, g):
            applied.append(("groups", g))

        def set_tuning(self, oz, wy):
            applied.append(("tuning", oz, wy))

        def set_graph(self, on):
            applied.append(("graph", on))

        def set_precond(self, m):
            applied.append(("precond", m))

    state = {}

    def cost(cfg):
        return (abs(cfg["groups"] - 16) + abs(cfg["wy_min"] - 96) / 10 + (cfg["oz_min"] != 4096) + (1 - cfg["graph"])
                + (cfg["precond"] != 64))

    real_apply = A.apply

    def fake_apply(ctx, cfg):
        state["cfg"] = dict(cfg)
        real_apply(ctx, cfg)

    class Ev:
        def __init__(self, **kw):
            self.t = 0.0

        def record(self):
            self.t = cost(state["cfg"]) * len(applied)

        def elapsed_time(self, other):
            return cost(state["cfg"])

    fake_torch = types.SimpleNamespace(cuda=types.SimpleNamespace(Event=Ev, synchronize=lambda: None))
    monkeypatch.setitem(sys.modules, "torch", fake_torch)
    monkeypatch.setattr(A, "apply", fake_apply)
    best, seen = A.tune(lambda: None, Ctx(), steps=1, warmup=0)
    assert best == {"groups": 16, "wy_min": 96, "oz_min": 4096, "graph": 1, "precond": 64}
    assert len(seen) <= 1 + sum(len(v) for v in A.CANDIDATES.values())


def test_ties_keep_the_defaults(monkeypatch):
    """A candidate faster by less than MIN_GAIN (run-to-run noise) does not replace the default."""
    state = {}

    class Ctx:
        def set_concurrency(self, g):
            pass

        def set_tuning(self, oz, wy):
            pass

        def set_graph(self, on):
            pass

        def set_precond(self, m):
            pass

    def cost(cfg):  # wy_min = off is 0.2 % faster, groups = 16 is 5 % faster
        c = 1000.0
        if cfg["wy_min"] == 1 << 30:
            c *= 0.998
        if cfg["groups"] == 16:
            c *= 0.95
        return c

    real_apply = A.apply

    def fake_apply(ctx, cfg):
        state["cfg"] = dict(cfg)
        real_apply(ctx, cfg)

    class Ev:
        def __init__(self, **kw):
            pass

        def record(self):
            pass

        def elapsed_time(self, other):
            return cost(state["cfg"])

    fake_torch = types.SimpleNamespace(cuda=types.SimpleNamespace(Event=Ev, synchronize=lambda: None))
    monkeypatch.setitem(sys.modules, "torch", fake_torch)
    monkeypatch.setattr(A, "apply", fake_apply)
    best, _ = A.tune(lambda: None, Ctx(), steps=1, warmup=0)
    assert best["groups"] == 16
    assert best["wy_min"] == A.DEFAULT["wy_min"]
