"""Autotuner host logic (no GPU): candidate grids, net samples, cache file."""
from orthoroute_gb300 import autotune as T


def test_candidates_cover_quarters_and_cta():
    assert T.candidates(304) == [("grid", 76), ("grid", 152), ("grid", 228), ("grid", 304), ("cta", 0)]
    assert T.candidates(2) == [("grid", 1), ("grid", 2), ("cta", 0)]


def test_net_samples():
    tasks = {f"N{i}": (0, i) for i in range(300)}
    dist = lambda s, d: d
    full = T.sample_full_nets(tasks, dist, 125, k=3)
    assert full == [(0, 299), (0, 298), (0, 297)]
    roi = T.sample_roi_nets(tasks, dist, 125, k=16)
    assert len(roi) == 16 and all(0 < d < 125 for _, d in roi) and len(set(roi)) == 16
    assert T.sample_roi_nets({"A": (0, 0)}, dist, 125) == []


def test_cache_roundtrip(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "tune.json"
    monkeypatch.setenv("ORTHOROUTE_GB300_TUNE_CACHE", str(path))
    assert T.cache_path() == str(path)
    t = T.Tuning(key="k", full_engine="grid", full_ctas=152, ms_per_search={"grid152": 1.0}, roi_lanes=2,
                 full_lanes=4, full_reuse=1, samples=3)
    T._store_cache(str(path), "k", t)
    T._store_cache(str(path), "k2", T.Tuning(key="k2", full_engine="cta", full_ctas=304))
    data = T._load_cache(str(path))
    assert set(data) == {"k", "k2"}
    back = T.Tuning(**data["k"])
    assert back == t
    path.write_text("not json")
    assert T._load_cache(str(path)) == {}
