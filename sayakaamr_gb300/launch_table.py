"""Per-kernel table of an ncu launch list (CSV from
`ncu --metrics gpu__time_duration.sum[,dram__bytes_read.sum,dram__bytes_write.sum] --csv`):
launches, total device time, share of the solve, and, when the DRAM
counters were captured, bytes moved per launch and the achieved DRAM
bandwidth against the measured copy peak.

    python -m sayakaamr_gb300.launch_table launches.csv [--peak GBPS] [--markdown]
"""
import argparse
import collections
import csv
import json
import os
import sys


def _num(v):
    return float(str(v).replace(",", ""))


def read_launches(path):
    """{launch id: {"name": kernel, metric: value}} from an ncu CSV"""
    with open(path, newline="") as f:
        lines = f.read().splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.startswith('"ID"'))
    rows = list(csv.DictReader(lines[start:]))
    out = collections.OrderedDict()
    for r in rows:
        lid = r["ID"]
        e = out.setdefault(lid, {"name": r["Kernel Name"]})
        try:
            val = _num(r["Metric Value"])
        except ValueError:
            continue
        unit = r.get("Metric Unit", "")
        if r["Metric Name"] == "gpu__time_duration.sum":
            val *= {"nsecond": 1e-9, "usecond": 1e-6, "msecond": 1e-3, "second": 1.0}.get(unit, 1e-9)
        elif r["Metric Name"].startswith("dram__bytes"):
            val *= {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6,
                    "GB": 1e9}.get(unit, 1.0)
        e[r["Metric Name"]] = val
    return out


def short(name):
    """kernel name without namespaces and argument lists"""
    n = name.split("(")[0].replace("void ", "")
    for pre in ("sayaka_gb300::<unnamed>::", "sayaka_gb300::"):
        n = n.replace(pre, "")
    return n.strip()


def table(launches, peak_gbs):
    agg = collections.OrderedDict()
    for e in launches.values():
        k = short(e["name"])
        a = agg.setdefault(k, dict(launches=0, seconds=0.0, bytes=0.0, has_bytes=False))
        a["launches"] += 1
        a["seconds"] += e.get("gpu__time_duration.sum", 0.0)
        if "dram__bytes_read.sum" in e:
            a["bytes"] += e["dram__bytes_read.sum"] + e.get("dram__bytes_write.sum", 0.0)
            a["has_bytes"] = True
    total = sum(a["seconds"] for a in agg.values()) or 1.0
    rows = []
    for k, a in sorted(agg.items(), key=lambda kv: -kv[1]["seconds"]):
        r = dict(kernel=k, launches=a["launches"], total_us=a["seconds"] * 1e6, share=a["seconds"] / total,
                 us_per_launch=a["seconds"] * 1e6 / a["launches"])
        if a["has_bytes"]:
            gbs = a["bytes"] / a["seconds"] / 1e9 if a["seconds"] > 0 else 0.0
            r.update(mb_per_launch=a["bytes"] / a["launches"] / 1e6, dram_gbs=gbs, frac_of_peak=gbs / peak_gbs)
        rows.append(r)
    return rows, total


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("csv")
    ap.add_argument("--peak", type=float, default=None, help="DRAM peak GB/s (default: MEASURED_PEAKS.json hbm_gbs)")
    ap.add_argument("--markdown", action="store_true")
    a = ap.parse_args(argv)
    peak = a.peak
    if peak is None:
        p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
        peak = float(json.load(open(p))["hbm_gbs"]) if os.path.exists(p) else 6800.0
    rows, total = table(read_launches(a.csv), peak)
    if not a.markdown:
        print(json.dumps(dict(total_us=total * 1e6, peak_gbs=peak, kernels=rows), indent=1))
        return
    print("| kernel | launches | total us | share | us/launch | DRAM MB/launch | DRAM GB/s | of peak |")
    print("|---|---|---|---|---|---|---|---|")
    for r in rows:
        print("| %s | %d | %.1f | %.1f%% | %.2f | %s | %s | %s |" % (
            r["kernel"], r["launches"], r["total_us"], 100 * r["share"], r["us_per_launch"],
            "%.2f" % r["mb_per_launch"] if "mb_per_launch" in r else "-",
            "%.0f" % r["dram_gbs"] if "dram_gbs" in r else "-",
            "%.2f" % r["frac_of_peak"] if "frac_of_peak" in r else "-"))
    print("\ntotal device time %.1f us (ncu, serialised launches); peak %.1f GB/s" % (total * 1e6, peak))


if __name__ == "__main__":
    sys.exit(main())
