"""Extracts statistics-grid shapes that the reference itself logged into a
golden fixture for hd_compute_stats.

For every input file, and for their union, the reference logs the non-empty
box ("MBR"), the point count, "StatsGridNumPointsPerCell", and what it derived
from them: the grid's "GridSize", its "CellDiagonalLength" and, per file, the
"Density" (src/run_hausdorff_distance.cu:150-200, src/geoms/mbr.h:288-296,
src/index/uniform_grid.h:222-244,695-705).  Its committed experiment logs
(expr/for_the_paper/logs/**.json) hold about 1,900 distinct such records from
its real runs.  This script keeps an even spread of them (2-D and 3-D, files
and unions) in tests/golden/log_grid_stats.json.

Run from the repository root in a container that has the reference sources:
    python tests/golden/make_log_grid_golden.py <reference root directory>
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
    seen = {}
    for path in logs:
        try:
            with open(path) as f:
                d = json.load(f)
        except (OSError, ValueError):
            continue
        inp = d.get("Input") if isinstance(d, dict) else None
        if not isinstance(inp, dict):
            continue
        files = [x for x in inp.get("Files", []) if isinstance(x, dict)]
        entries = [("file", x, x.get("NumPoints")) for x in files]
        if files:
            entries.append(("union", inp, sum(x.get("NumPoints", 0) for x in files)))
        for kind, x, n in entries:
            g = x.get("Grid")
            if not isinstance(g, dict) or "MBR" not in x or x.get("StatsGridNumPointsPerCell") is None:
                continue
            lower = [m["Lower"] for m in x["MBR"]]
            upper = [m["Upper"] for m in x["MBR"]]
            key = (tuple(lower), tuple(upper), n, x["StatsGridNumPointsPerCell"], kind)
            if key in seen:
                continue
            rec = {"log": os.path.relpath(path, root), "kind": kind, "lower": lower,
                   "upper": upper, "n": n, "n_points_cell": x["StatsGridNumPointsPerCell"],
                   "grid_size": g["GridSize"], "cell_diagonal": g["CellDiagonalLength"]}
            if kind == "file":
                rec["density"] = x["Density"]
            seen[key] = rec
    recs = sorted(seen.values(), key=lambda r: (len(r["lower"]), r["kind"], r["n"], r["log"]))
    groups = {}
    for r in recs:
        groups.setdefault((len(r["lower"]), r["kind"]), []).append(r)
    out = []
    for _, g in sorted(groups.items()):
        out += g[::max(1, len(g) // 50)]
    with open(os.path.join(HERE, "log_grid_stats.json"), "w") as f:
        f.write('{"generator": "tests/golden/make_log_grid_golden.py",\n'
                ' "source": "expr/for_the_paper/logs/**.json, MBR/NumPoints/Grid/Density",\n'
                f' "distinct_records_in_logs": {len(recs)},\n "records": [\n')
        f.write(",\n".join(json.dumps(r, separators=(",", ":")) for r in out))
        f.write("\n]}\n")
    print(f"{len(recs)} distinct records, {len(out)} kept")


if __name__ == "__main__":
    main()
