"""CPU tests: the key under which a tuned batch plan is kept (preset mix and
GPU) and the JSON store of plans."""

import pytest

from nebc7_gb300 import BatchTexture, PlanStore, plan_key
from nebc7_gb300._native import Settings


def _tex(w, h, st):
    return BatchTexture(0, 0, None, w * 4, w, h, Settings(*st))


def test_plan_key_is_the_mix_per_preset_and_the_device():
    a = [_tex(256, 256, (1, 9, 1, 1, 0, 0)), _tex(64, 64, (0, 0, 1, 1, 0, 0))]
    k = plan_key(a, "GB300")
    assert k.startswith("GB300|")
    # the order of the textures does not matter, nor a size within the same power of two of blocks
    assert plan_key(a[::-1], "GB300") == k
    b = [_tex(256, 300, (1, 9, 1, 1, 0, 0)), _tex(64, 64, (0, 0, 1, 1, 0, 0))]
    assert plan_key(b, "GB300") == k
    # another preset mix, another size class or another GPU is another key
    assert plan_key([_tex(256, 256, (1, 9, 1, 1, 1, 0)), a[1]], "GB300") != k
    assert plan_key([_tex(1024, 1024, (1, 9, 1, 1, 0, 0)), a[1]], "GB300") != k
    assert plan_key(a, "B200") != k
    # textures of one preset add up
    assert plan_key([_tex(128, 128, (1, 9, 1, 1, 0, 0))] * 4 + [a[1]], "GB300") == k


def test_plan_store_round_trip(tmp_path):
    store = PlanStore(tmp_path / "plans.json")
    assert store.get("k") is None
    store.put("k", {"schedule": "grouped", "staged": 1, "ctas_per_sm": 2, "ms": 3.5})
    store.put("j", {"schedule": "mixed", "staged": False, "ctas_per_sm": 0})
    again = PlanStore(tmp_path / "plans.json")
    assert again.get("k") == {"schedule": "grouped", "staged": True, "ctas_per_sm": 2}
    assert again.get("j") == {"schedule": "mixed", "staged": False, "ctas_per_sm": 0}
    assert not (tmp_path / "plans.json.tmp").exists()
