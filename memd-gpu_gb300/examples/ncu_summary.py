"""Summary of an ncu launch list (--csv --log-file) of one decomposition.

    python memd-gpu_gb300/examples/ncu_summary.py launches.csv [--form mixed] [--traffic-json out.json]
        [--source "<the capture command>"]

Prints a markdown table per kernel (launches, total device time, share,
DRAM bytes per launch when the capture has dram__bytes_read.sum /
dram__bytes_write.sum) and per stage of the sift (project, compact, factor,
solve, eval).  With --traffic-json it merges "<form>:<stage>" entries --
DRAM bytes per launch averaged over every launch of the stage -- into that
file, the format bench.py reads for the roofline's "traffic" figure.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import re
from collections import OrderedDict

# kernel name prefix -> sift stage (the stage names of the plan's profile)
STAGES = (
    ("k_split_tf32", "project"),
    ("k_project", "project"),
    ("k_compact", "compact"),
    ("k_mirror", "compact"),
    ("k_factor", "factor"),
    ("k_solve", "solve"),
    ("k_mean_cum", "eval"),
    ("k_eval", "eval"),
    ("k_amp", "stop"),
    ("k_stop", "stop"),
    ("k_decide", "stop"),
    ("k_apply", "stop"),
)


def short_name(full: str) -> str:
    """'void k_solve_fwd<dd, float2, 1, 0, 0>(...)' -> 'k_solve_fwd<dd, float2, 1, 0, 0>'."""
    s = full
    if s.startswith("void "):
        s = s[5:]
    depth = 0
    for i, ch in enumerate(s):
        if ch == "<":
            depth += 1
        elif ch == ">":
            depth -= 1
        elif ch == "(" and depth == 0:
            return s[:i]
    return s


def stage_of(name: str) -> str:
    for pre, st in STAGES:
        if name.startswith(pre):
            return st
    return "other"


def read_launches(path: str):
    """{launch id: {"kernel": short name, metric: value}} in launch order."""
    text = open(path).read()
    start = text.find('"ID"')
    if start < 0:
        raise SystemExit(f"{path}: no ncu CSV header")
    rows = csv.DictReader(io.StringIO(text[start:]))
    out: "OrderedDict[str, dict]" = OrderedDict()
    for r in rows:
        d = out.setdefault(r["ID"], {"kernel": short_name(r["Kernel Name"])})
        v = r["Metric Value"].replace(",", "")
        try:
            d[r["Metric Name"]] = float(v)
        except ValueError:
            pass
    return list(out.values())


def summarise(launches):
    per = OrderedDict()
    for l in launches:
        k = per.setdefault(l["kernel"], {"launches": 0, "ns": 0.0, "bytes": 0.0, "has_bytes": False})
        k["launches"] += 1
        k["ns"] += l.get("gpu__time_duration.sum", 0.0)
        if "dram__bytes_read.sum" in l or "dram__bytes_write.sum" in l:
            k["has_bytes"] = True
            k["bytes"] += l.get("dram__bytes_read.sum", 0.0) + l.get("dram__bytes_write.sum", 0.0)
    stages = OrderedDict()
    for name, k in per.items():
        st = stages.setdefault(stage_of(name), {"launches": 0, "ns": 0.0, "bytes": 0.0, "has_bytes": False})
        st["launches"] += k["launches"]
        st["ns"] += k["ns"]
        st["bytes"] += k["bytes"]
        st["has_bytes"] |= k["has_bytes"]
    return per, stages


def table(rows, total_ns, label):
    out = [f"| {label} | launches | total ms | share | DRAM bytes per launch |", "|---|---|---|---|---|"]
    for name, k in sorted(rows.items(), key=lambda kv: -kv[1]["ns"]):
        b = f"{k['bytes'] / k['launches']:.4g}" if k["has_bytes"] else "-"
        out.append(f"| `{name}` | {k['launches']} | {k['ns'] / 1e6:.3f} | {100 * k['ns'] / max(total_ns, 1):.1f}% | {b} |")
    n = sum(k["launches"] for k in rows.values())
    out.append(f"| total | {n} | {total_ns / 1e6:.3f} | | |")
    return "\n".join(out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("csv")
    ap.add_argument("--form", default="mixed")
    ap.add_argument("--traffic-json")
    ap.add_argument("--source", default="")
    a = ap.parse_args()
    launches = read_launches(a.csv)
    per, stages = summarise(launches)
    total = sum(k["ns"] for k in per.values())
    print(table(per, total, "kernel"))
    print()
    print(table(stages, total, "stage"))
    if a.traffic_json:
        data = {}
        if os.path.exists(a.traffic_json):
            data = json.load(open(a.traffic_json))
        for st, k in stages.items():
            if k["has_bytes"] and st != "other":
                data[f"{a.form}:{st}"] = {"bytes_per_launch": k["bytes"] / k["launches"], "launches": k["launches"],
                                          "source": a.source}
        with open(a.traffic_json, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main()
