"""The autotuner's table fit (no GPU): the threshold minimises the sweep's
total time and the index preference follows total index time."""
from hausdorffdistance_gb300 import autotune


def test_fit_picks_cost_minimising_threshold(tmp_path):
    rows = [
        {"ratio": 1.0, "pairs": 1e6, "eb": 1.0, "lbvh": 5.0, "grid": 6.0},
        {"ratio": 10.0, "pairs": 1e8, "eb": 2.0, "lbvh": 3.0, "grid": 4.0},
        {"ratio": 100.0, "pairs": 1e10, "eb": 50.0, "lbvh": 3.0, "grid": 9.0},
        {"ratio": 1000.0, "pairs": 1e12, "eb": 500.0, "lbvh": 4.0, "grid": 2.0},
    ]
    p = autotune.fit(rows)
    assert p["prefer_grid"] is False  # lbvh total 15 < grid total 21
    assert p["total_ms_chosen"] == 1.0 + 2.0 + 3.0 + 4.0
    assert p["total_ms_oracle_choice"] == 1.0 + 2.0 + 3.0 + 2.0
    autotune.write_table(p, str(tmp_path / "t.h"))
    text = (tmp_path / "t.h").read_text()
    assert "HD_TUNED_EB_RATIO" in text and "HD_TUNED_PREFER_GRID 0" in text
    assert "HD_TUNED_INDEX_MIN_PAIRS" in text and "HD_TUNED_EB_SMALL_PAIRS" in text
