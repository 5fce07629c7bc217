"""Extracts percentile tables that the reference itself logged into a golden
fixture for the statistics grid's "Histogram" entry.

The reference writes, for every input file and for their union, the
percentile table of points per non-empty statistics-grid cell as printed by
HdrHistogram_c (src/index/uniform_grid.h:675-693, src/running_stats.h:106-140);
its committed experiment logs (expr/for_the_paper/logs/**.json) hold about two
thousand distinct tables from its real runs.  This script keeps a varied
subset (every degenerate table, every table with values of 2048 or more, where
HdrHistogram's three significant figures round values into buckets, and an
even spread of the rest by length) with the log each came from, in
tests/golden/hdr_percentiles.json.

Run from the repository root in a container that has the reference sources:
    python tests/golden/make_hdr_golden.py <reference root directory>
"""
from __future__ import annotations

import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    root = sys.argv[1]
    logs = sorted(glob.glob(os.path.join(root, "expr", "for_the_paper", "logs", "**", "*.json"),
                            recursive=True))
    tables = {}
    for path in logs:
        try:
            with open(path) as f:
                d = json.load(f)
        except (OSError, ValueError):
            continue
        inp = d.get("Input", {}) if isinstance(d, dict) else {}
        grids = [(f"Files[{i}]", x.get("Grid")) for i, x in enumerate(inp.get("Files", []))
                 if isinstance(x, dict)]
        grids.append(("Input", inp.get("Grid")))
        for where, g in grids:
            if not isinstance(g, dict) or not g.get("Histogram"):
                continue
            rows = tuple((r["value"], r["percentile"], r["count"]) for r in g["Histogram"])
            if rows not in tables:
                tables[rows] = (os.path.relpath(path, root), where)
    keys = sorted(tables, key=lambda r: (len(r), r))
    degenerate = [r for r in keys if r[-1][2] < 2]
    big = [r for r in keys if r[-1][2] >= 2 and max(v for v, _, _ in r) >= 2048]
    rest = [r for r in keys if r[-1][2] >= 2 and max(v for v, _, _ in r) < 2048]
    pick = degenerate + big[::max(1, len(big) // 60)] + rest[::max(1, len(rest) // 80)]
    out = [{"log": tables[r][0], "grid": tables[r][1], "rows": [list(x) for x in r]}
           for r in sorted(pick, key=lambda r: (len(r), r))]
    with open(os.path.join(HERE, "hdr_percentiles.json"), "w") as f:
        f.write('{"generator": "tests/golden/make_hdr_golden.py",\n'
                ' "source": "expr/for_the_paper/logs/**.json, Grid.Histogram",\n'
                f' "distinct_tables_in_logs": {len(tables)},\n "tables": [\n')
        f.write(",\n".join(json.dumps(t, separators=(",", ":")) for t in out))
        f.write("\n]}\n")
    print(f"{len(tables)} distinct tables, {len(out)} kept")


if __name__ == "__main__":
    main()
