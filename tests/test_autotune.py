"""The autotuner's table fit (no GPU): every threshold minimises the sweep's
total time; the grid is chosen from the outside / skew statistics."""
from hausdorffdistance_gb300 import autotune


def test_fit_picks_cost_minimising_thresholds(tmp_path):
    rows = [
        # small: EB wins
        {"ratio": 1.0, "pairs": 1e6, "outside": 0.0, "skew": 1.0, "eb": 1.0, "lbvh": 5.0, "grid": 6.0},
        # duplicated data: tiny ratio, EB wins although the problem is large
        {"ratio": 8.0, "pairs": 1e9, "outside": 0.0, "skew": 900.0, "eb": 2.0, "lbvh": 3.0, "grid": 4.0},
        # uniform, no outliers: grid wins
        {"ratio": 1000.0, "pairs": 1e10, "outside": 0.0, "skew": 1.1, "eb": 50.0, "lbvh": 3.0,
         "grid": 2.0},
        # outliers: grid loses badly
        {"ratio": 1000.0, "pairs": 1e10, "outside": 0.03, "skew": 1.2, "eb": 50.0, "lbvh": 3.0,
         "grid": 30.0},
        # clustered: grid loses badly
        {"ratio": 8000.0, "pairs": 1e12, "outside": 0.0, "skew": 40.0, "eb": 500.0, "lbvh": 4.0,
         "grid": 20.0},
    ]
    p = autotune.fit(rows)
    assert p["total_ms_chosen"] == p["total_ms_oracle_choice"] == 1.0 + 2.0 + 2.0 + 3.0 + 4.0
    assert [autotune.choose(r, p["eb_small_pairs"], p["eb_ratio"], p["grid_max_outside"],
                            p["grid_max_skew"]) for r in rows] == ["eb", "eb", "grid", "lbvh", "lbvh"]
    autotune.write_table(p, str(tmp_path / "t.h"))
    text = (tmp_path / "t.h").read_text()
    for name in ("EB_RATIO", "INDEX_MIN_PAIRS", "EB_SMALL_PAIRS", "EB_SAMPLE_MAX_PAIRS",
                 "GRID_MAX_OUTSIDE", "GRID_MAX_SKEW"):
        assert f"HD_TUNED_{name} " in text


def test_batch_fit_and_table(tmp_path):
    rows = [{"batch_small_rows": s, "batch_chunk": c, "ms": 10.0 + abs(s - autotune.BATCH_SMALL_ROWS[1]) / 100 + c / 10}
            for s in autotune.BATCH_SMALL_ROWS for c in autotune.BATCH_CHUNKS]
    p = autotune.fit_batch(rows)
    assert p["batch_small_rows"] == autotune.BATCH_SMALL_ROWS[1]
    assert p["batch_chunk"] == min(autotune.BATCH_CHUNKS)
    sel = {"eb_ratio": 0, "eb_small_pairs": 0, "index_min_pairs": 0,
           "eb_sample_max_pairs": 1e10, "grid_max_outside": 0.002, "grid_max_skew": 2.0}
    autotune.write_table({**sel, **p}, str(tmp_path / "t.h"))
    text = (tmp_path / "t.h").read_text()
    assert f"HD_TUNED_BATCH_SMALL_ROWS {autotune.BATCH_SMALL_ROWS[1]}" in text
    assert f"HD_TUNED_BATCH_CHUNK {min(autotune.BATCH_CHUNKS)}" in text
    # Without a batch sweep the table keeps the defaults.
    autotune.write_table(sel, str(tmp_path / "u.h"))
    assert "HD_TUNED_BATCH_SMALL_ROWS 8192" in (tmp_path / "u.h").read_text()


def test_read_table_round_trip(tmp_path):
    sel = {"eb_ratio": 0.5, "eb_small_pairs": 1e6, "index_min_pairs": 4e6,
           "eb_sample_max_pairs": 1e10, "grid_max_outside": 0.002, "grid_max_skew": 2.0}
    autotune.write_table(sel, str(tmp_path / "t.h"))
    got = autotune.read_table(str(tmp_path / "t.h"))
    assert {k: got[k] for k in sel} == sel
    # Schedule values not swept keep what the table holds.
    autotune.write_table({**sel, "batch_chunk": 16, "lbvh_budget": 512}, str(tmp_path / "u.h"))
    got = autotune.read_table(str(tmp_path / "u.h"))
    assert got["batch_chunk"] == 16 and got["lbvh_budget"] == 512


def test_budget_fit_and_table(tmp_path):
    rows = [{"case": c, "lbvh_budget": b, "ms": t}
            for c, ts in (("x", {128: 3.0, 256: 2.0, 512: 2.5}), ("y", {128: 1.0, 256: 1.5, 512: 1.0}))
            for b, t in ts.items()]
    p = autotune.fit_budget(rows)
    assert p["lbvh_budget"] == 256 and p["lbvh_budget_total_ms"] == 3.5
    sel = {"eb_ratio": 0, "eb_small_pairs": 0, "index_min_pairs": 0,
           "eb_sample_max_pairs": 1e10, "grid_max_outside": 0.002, "grid_max_skew": 2.0}
    autotune.write_table({**sel, **p}, str(tmp_path / "t.h"))
    assert "HD_TUNED_LBVH_BUDGET 256" in (tmp_path / "t.h").read_text()
