"""The batched form's tuner (serving.autotune): each candidate timed after its own
warm-up, the one with the lowest median stored per key in a JSON cache, a cache
hit running only the stored candidate.  Host logic only (a fake batch and clock)."""

import json

from bone_morphometry_gb300 import serving as SV
from bone_morphometry_gb300._lib import BM_SITES_AUTO, BM_SITES_CHAINS, BM_SITES_SPHERES


class FakeBatch:
    """Pretends each candidate takes cost[(w, m, c)] seconds on a fake clock."""

    def __init__(self, cost):
        self.cost = cost
        self.now = 0.0
        self.calls = []

    def clock(self):
        return self.now

    def run(self, *cand):
        self.calls.append(cand)
        self.now += self.cost[cand]
        return ["result"]


CANDS = ((2, BM_SITES_AUTO, 32, True), (4, BM_SITES_SPHERES, 64, False), (8, BM_SITES_CHAINS, 32, True))


def test_picks_the_fastest_and_persists(tmp_path):
    path = str(tmp_path / "sub" / "tuning.json")
    fb = FakeBatch({CANDS[0]: 0.30, CANDS[1]: 0.10, CANDS[2]: 0.20})
    res, t = SV.autotune(fb.run, "gpu|mix", path, CANDS, clock=fb.clock)
    assert res == ["result"]
    assert t.setting() == (4, BM_SITES_SPHERES, 64, False)
    assert abs(t.batch_ms - 100.0) < 1e-9 and not t.from_cache
    assert fb.calls == [c for c in CANDS for _ in range(4)]  # each candidate: a warm-up, then three timed runs
    stored = json.load(open(path))
    assert stored == {"gpu|mix": {"workers": 4, "site_method": BM_SITES_SPHERES, "fill_tile_rows": 64,
                                  "concurrent_phases": False, "batch_ms": 100.0}}


def test_cache_hit_runs_only_the_stored_candidate(tmp_path):
    path = str(tmp_path / "tuning.json")
    fb = FakeBatch({CANDS[0]: 0.3, CANDS[1]: 0.2, CANDS[2]: 0.1})
    SV.autotune(fb.run, "k", path, CANDS, clock=fb.clock)
    fb.calls.clear()
    res, t = SV.autotune(fb.run, "k", path, CANDS, clock=fb.clock)
    assert t.from_cache and t.setting() == CANDS[2]
    assert fb.calls == [CANDS[2]] and res == ["result"]
    # another key tunes again and keeps the first entry
    fb.calls.clear()
    SV.autotune(fb.run, "k2", path, CANDS, clock=fb.clock)
    assert len(fb.calls) == 12 and set(json.load(open(path))) == {"k", "k2"}


def test_median_not_a_lucky_run(tmp_path):
    """A candidate with one fast outlier loses to one that is steadily faster."""
    seq = {CANDS[0]: [0.5, 0.05, 0.5, 0.5], CANDS[1]: [0.2, 0.2, 0.2, 0.2], CANDS[2]: [0.3, 0.3, 0.3, 0.3]}

    class Seq(FakeBatch):
        def run(self, *cand):
            self.calls.append(cand)
            self.now += seq[cand].pop(0)
            return ["r"]

    fb = Seq({})
    _, t = SV.autotune(fb.run, "k", str(tmp_path / "t.json"), CANDS, clock=fb.clock)
    assert (t.workers, t.site_method) == (4, BM_SITES_SPHERES)


def test_retune_and_unreadable_cache(tmp_path):
    path = tmp_path / "tuning.json"
    path.write_text("{not json")
    fb = FakeBatch({CANDS[0]: 0.1, CANDS[1]: 0.2, CANDS[2]: 0.3})
    _, t = SV.autotune(fb.run, "k", str(path), CANDS, clock=fb.clock)
    assert (t.workers, t.from_cache) == (2, False)
    fb.cost[CANDS[0]] = 0.5
    _, t = SV.autotune(fb.run, "k", str(path), CANDS, retune=True, clock=fb.clock)
    assert (t.workers, t.site_method) == (4, BM_SITES_SPHERES)
    assert json.load(open(path))["k"]["workers"] == 4


def test_entry_without_every_setting_is_tuned_again(tmp_path):
    path = tmp_path / "tuning.json"
    path.write_text(json.dumps({"k": {"workers": 4, "site_method": 0, "concurrent_phases": True, "batch_ms": 9.0}}))
    fb = FakeBatch({CANDS[0]: 0.3, CANDS[1]: 0.1, CANDS[2]: 0.2})
    _, t = SV.autotune(fb.run, "k", str(path), CANDS, clock=fb.clock)
    assert not t.from_cache and t.setting() == CANDS[1]


def test_no_candidates(tmp_path):
    import pytest

    with pytest.raises(ValueError, match="at least one candidate"):
        SV.autotune(lambda *c: None, "k", str(tmp_path / "t.json"), ())


def test_mix_signature_buckets():
    a = SV.mix_signature([(96, 100, 120), (384, 300, 200)])
    b = SV.mix_signature([(200, 300, 384), (120, 100, 96)])  # order and axis order do not matter
    assert a == b
    assert SV.mix_signature([(128, 128, 128)] * 64) != SV.mix_signature([(128, 128, 128)] * 8)
    assert SV.mix_signature([(128, 128, 128)]) != SV.mix_signature([(256, 256, 256)])
    assert SV.mix_signature([]) == "empty"


def test_default_cache_path(monkeypatch, tmp_path):
    monkeypatch.setenv("BM_TUNE_CACHE", str(tmp_path / "x.json"))
    assert SV.tuning_cache_path() == str(tmp_path / "x.json")
    monkeypatch.delenv("BM_TUNE_CACHE")
    assert SV.tuning_cache_path().endswith("batch_tuning.json")
