"""Host logic of the Radon tile shapes, without a GPU: the FP16 method's slab re-layout in
BandDetect._pick_method and the autotuner's decision cache holding the tile shape, against a
fake device plan that models ebsd_plan_get_tile / ebsd_plan_set_tile."""
import pytest

import pyebsdindex_gb300 as pg
from pyebsdindex_gb300 import _lib


class FakePlan:
    """A slab plan: FP16 storage fits from `fp16_from` slabs on; `single` says whether the
    one-tile kernel takes the plan (then FP16 runs there whatever the slabs)."""

    device = 0

    def __init__(self, slabs=9, slabs_max=11, fp16_from=10, single=False):
        self.slabs, self.slabs_max, self.fp16_from, self.single = slabs, slabs_max, fp16_from, single
        self.tile_mode, self.calls, self.ppp = 0, [], 0

    def get_tile(self):
        return {"tile": 1 if self.single and self.tile_mode != 2 else 2, "patterns_per_pass": self.ppp,
                "slabs": self.slabs, "slab_columns": (180 + self.slabs - 1) // self.slabs, "slabs_min": 9,
                "slabs_max": self.slabs_max, "single_fits": int(self.single),
                "slabs_fp16": int(self.slabs >= self.fp16_from)}

    def set_tile(self, tile, slabs=0):
        if tile == 1 and not self.single:
            raise RuntimeError("ebsd_plan_set_tile failed: plan shape not supported by this method (code -5)")
        if slabs and not 9 <= slabs <= self.slabs_max:
            raise RuntimeError("ebsd_plan_set_tile failed: plan shape not supported by this method (code -5)")
        self.calls.append((tile, slabs))
        self.tile_mode = tile
        self.slabs = slabs or 9

    def set_patterns_per_pass(self, ppp):
        self.ppp = ppp

    def supported(self, method, dtype=None):
        if method == "fused16":
            if dtype not in (None, _lib.EBSD_U8, _lib.EBSD_U16):
                return self.single
            return self.single or self.slabs >= self.fp16_from
        return True


def detector():
    return pg.BandDetect(patDim=(240, 240), nRho=360, nTheta=180, tSigma=1.0, rSigma=1.0, nBands=10)


def test_fp16_relays_the_slabs_to_the_widest_that_take_it():
    plan = FakePlan()
    assert detector()._pick_method(plan, "fused16", _lib.EBSD_U16) == "fused16"
    assert plan.slabs == 10 and plan.calls == [(0, 10)]


def test_fp16_on_a_plan_whose_slabs_never_take_it_restores_the_slabs():
    plan = FakePlan(fp16_from=99)
    assert detector()._pick_method(plan, "fused16", _lib.EBSD_U16) == "plain"
    assert plan.slabs == 9 and plan.calls[-1] == (0, 9)


def test_fp16_leaves_one_tile_plans_and_float_input_alone():
    plan = FakePlan(single=True)
    assert detector()._pick_method(plan, "fused16", _lib.EBSD_U8) == "fused16"
    assert plan.calls == []
    plan = FakePlan()
    assert detector()._pick_method(plan, "fused16", _lib.EBSD_F32) == "plain"
    assert plan.calls == []  # float32 patterns have no FP16 slab kernel: nothing is re-laid


def test_fp32_methods_never_relay():
    plan = FakePlan()
    assert detector()._pick_method(plan, "fused", _lib.EBSD_U16) == "fused"
    assert plan.calls == []


def test_cached_tile_decision_is_applied_without_timing(tmp_path, monkeypatch):
    from pyebsdindex_gb300 import tuning
    bd = detector()
    plan = FakePlan()
    monkeypatch.setattr(bd, "_device_plan", lambda gpu_id=None: plan)
    monkeypatch.setattr(bd, "_tuning_key", lambda p, m, dt: "key")
    monkeypatch.setattr(bd, "_pick_method", lambda p, m, dt=None: "fused")
    path = tmp_path / "tuning.json"
    tuning.TuningCache(path).put("key", {"patterns_per_pass": 1, "tile": 2, "slabs": 11, "timed_patterns": 64})
    torch = pytest.importorskip("torch")
    sample = torch.zeros((4, 240, 240), dtype=torch.float32)
    assert bd.autotune(sample, method="fused", cache=path) == 1
    assert plan.calls == [(2, 11)] and bd.tuned["cached"] and bd.tuned["slabs"] == 11


def test_cached_tile_decision_the_plan_refuses_is_tuned_afresh(tmp_path, monkeypatch):
    from pyebsdindex_gb300 import tuning
    bd = detector()
    plan = FakePlan(slabs_max=10)
    timed = []

    def autotune(ptr, dt, n, m, stream=0):
        timed.append(n)
        plan.set_tile(2, 10)
        return 1
    plan.autotune = autotune
    monkeypatch.setattr(bd, "_device_plan", lambda gpu_id=None: plan)
    monkeypatch.setattr(bd, "_tuning_key", lambda p, m, dt: "key")
    monkeypatch.setattr(bd, "_pick_method", lambda p, m, dt=None: "fused")
    path = tmp_path / "tuning.json"
    tuning.TuningCache(path).put("key", {"patterns_per_pass": 1, "tile": 2, "slabs": 11})
    torch = pytest.importorskip("torch")
    sample = torch.zeros((4, 240, 240), dtype=torch.float32)
    # the stored 11 slabs are beyond this plan's range: the decision is timed and rewritten (the
    # sample stays on the host: the fake plan reads nothing)
    monkeypatch.setattr(torch.Tensor, "to", lambda self, *a, **k: self)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda dev=None: type("S", (), {"cuda_stream": 0})())
    assert bd.autotune(sample, method="fused", cache=path) == 1
    assert timed == [4] and not bd.tuned["cached"]
    assert tuning.TuningCache(path).get("key")["slabs"] == 10
