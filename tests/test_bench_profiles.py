"""bench.py reads per-kernel figures from the committed ncu summaries in
profiles/ (DRAM bytes per unit for the roofline's `traffic`, issue and
tensor-pipe activity beside the fractions).  Every summary it reads must hold
the figures it reads, or the JSON line would carry nulls."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
bench = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(bench)

NEEDED = {
    "morton_sort": ["dram_bytes_per_unit"],
    "lbvh_build": ["dram_bytes_per_unit", "issue_active"],
    "lbvh_query": ["dram_bytes_per_unit", "issue_active"],
    "eb_main": ["issue_active"],
    "bf16_rowmin": ["dram_bytes_per_unit", "tensor_pipe_active"],
    "batch": ["dram_bytes_per_unit", "issue_active"],
}


@pytest.mark.parametrize("tag", sorted(NEEDED))
def test_profile_summaries_hold_the_figures_bench_reads(tag):
    fig = bench.profile_figures(tag)
    for key in NEEDED[tag]:
        assert key in fig and fig[key] > 0, (tag, key)
    # Each summary names the command that produced it.
    text = open(os.path.join(ROOT, "profiles", f"{tag}.txt")).read()
    assert "ncu " in text and "--clock-control none" in text


def test_traffic_scales_with_units():
    per_unit = bench.profile_figures("lbvh_query")["dram_bytes_per_unit"]
    assert bench.traffic_from_profiles("lbvh_query", 2e7) == pytest.approx(per_unit * 2e7)
    assert bench.traffic_from_profiles("no_such_profile", 10.0) is None


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(os.path.join(ROOT, "profiles"))
                                        if f.endswith(".txt")))
def test_every_profile_names_its_command(name):
    """Each summary gives the ncu command that made it, with the clocks left
    alone (--clock-control none), and no raw report is committed beside it."""
    text = open(os.path.join(ROOT, "profiles", name)).read()
    assert "ncu " in text and "--clock-control none" in text
    assert not any(f.endswith((".ncu-rep", ".nsys-rep", ".qdrep"))
                   for f in os.listdir(os.path.join(ROOT, "profiles")))


def test_lbvh_algorithmic_bytes_follow_their_definitions():
    """Sort: per set the points read twice, two 16-byte key/index passes, the
    sorted points written; build: 2 n/16 nodes of 32 B per set; query: the
    queries' coordinates, 32 B per visited node, the visited leaves' points."""
    class Counts:
        visited_nodes = 1_000
        visited_leaves = 300

    n = 10_000_000
    phases = dict((tag, b) for tag, b, _ in
                  bench._lbvh_phases(n, n, 3, True, Counts, [0.8, 0.2, 0.0, 0.4]))
    assert phases["morton_sort"] == 2 * n * (12 * 2 + 32 + 12) == 1_360_000_000
    assert phases["lbvh_build"] == 2 * (2 * (n // 16)) * 32
    assert phases["lbvh_query"] == 2 * n * 12 + 1_000 * 32 + 300 * 16 * 12
    directed = dict((tag, b) for tag, b, _ in
                    bench._lbvh_phases(n, n // 2, 2, False, Counts, [0.8, 0.2, 0.0, 0.4]))
    assert directed["lbvh_query"] == n * 8 + 1_000 * 32 + 300 * 16 * 8
