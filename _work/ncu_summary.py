"""Summarizes an ncu launch list (--metrics gpu__time_duration.sum --csv)
into per-kernel launches, total time and share.  Usage:
    python -m aphros_gb300.ncu_summary launches.csv
"""
import csv
import re
import sys
from collections import defaultdict


def short(name):
    name = re.sub(r"\(.*", "", name)
    name = name.replace("unnamed>::", "").replace("aphgpu::", "")
    return name.strip()


def main(path):
    rows = []
    with open(path) as f:
        lines = [l for l in f if l.startswith('"')]
    for r in csv.DictReader(lines):
        if r.get("Metric Name") != "gpu__time_duration.sum":
            continue
        v = float(r["Metric Value"].replace(",", ""))
        unit = r["Metric Unit"]
        ns = v * {"ns": 1, "us": 1e3, "usecond": 1e3, "ms": 1e6, "msecond": 1e6}.get(unit, 1)
        rows.append((short(r["Kernel Name"]), r["Grid Size"], ns))
    agg = defaultdict(lambda: [0, 0.0])
    for name, grid, ns in rows:
        agg[name][0] += 1
        agg[name][1] += ns
    total = sum(v[1] for v in agg.values())
    print("%d launches, %.3f ms total device time" % (len(rows), total / 1e6))
    print("%-40s %8s %12s %7s" % ("kernel", "launches", "total ms", "share"))
    for name, (n, t) in sorted(agg.items(), key=lambda kv: -kv[1][1]):
        print("%-40s %8d %12.3f %6.1f%%" % (name, n, t / 1e6, 100 * t / total))


if __name__ == "__main__":
    main(sys.argv[1])
