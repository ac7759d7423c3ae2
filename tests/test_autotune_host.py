"""The autotuner's host logic (wannier90_gb300/autotune.py) with the GPU timing replaced by
a fixed table: which candidates each width gets, the fastest one chosen with its engine
options, the per-process cache, and the JSON table."""
import json

import pytest

from wannier90_gb300 import autotune as AT


@pytest.fixture(autouse=True)
def _fresh_cache():
    AT._CACHE.clear()
    yield
    AT._CACHE.clear()


def test_candidates_by_width():
    assert AT.candidates_for(4) == ["fp64", "tensor", "tensor_fp64exp", "tensor_cta"]
    assert AT.candidates_for(16) == ["fp64", "tensor", "tensor_fp64exp", "tensor_cta"]
    assert AT.candidates_for(24) == ["fp64", "tensor", "tensor_fp64exp", "tensor_cta", "tensor_smemexp"]
    assert AT.candidates_for(32)[-1] == "tensor_smemexp"
    assert AT.candidates_for(64) == ["fp64", "tensor", "tensor_fp64exp"]
    assert AT.candidates_for(128) == ["fp64", "tensor", "tensor_fp64exp"]
    assert AT.candidates_for(129) == ["fp64"]
    for w in (4, 24, 64, 129):
        assert all(n in AT.CANDIDATES for n in AT.candidates_for(w))


def test_fastest_candidate_is_chosen_and_cached(monkeypatch):
    fake = {"fp64": 3.0, "tensor": 1.0, "tensor_fp64exp": 2.0, "tensor_cta": 0.5, "tensor_smemexp": 0.7}
    calls = []

    def timed(p, opts, iters):
        name = next(n for n, o in AT.CANDIDATES.items() if o == opts)
        calls.append(name)
        assert p.num_wann == 24 and iters == 12
        return fake[name]

    monkeypatch.setattr(AT, "_time_variant", timed)
    res = AT.tune(24)
    assert res["choice"] == "tensor_cta"
    assert res["options"] == AT.CANDIDATES["tensor_cta"] and res["tensor"] == 1
    assert sorted(calls) == sorted(AT.candidates_for(24))
    assert AT.options(24) == AT.CANDIDATES["tensor_cta"] and AT.choose_tensor(24) == 1
    assert len(calls) == 5          # later calls come from the cache


def test_widest_problems_need_no_timing(monkeypatch, tmp_path):
    monkeypatch.setattr(AT, "_time_variant", lambda *a: pytest.fail("timed a single-candidate width"))
    res = AT.tune(200)
    assert res == {"choice": "fp64", "options": {"gpu_tensor": 0}, "tensor": 0, "times": {"fp64": None}}
    path = tmp_path / "sub" / "tune.json"
    out = AT.table([200, 200], str(path))
    assert list(out) == [200]
    assert json.loads(path.read_text())["200"]["choice"] == "fp64"
