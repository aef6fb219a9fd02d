"""Per-launch figures of an ncu capture, in the machine-readable form bench.py reads.

bench.py reports two numbers it cannot measure inside its own timed region: the
DRAM bytes of one association launch (roofline.traffic) and the warp instructions
the association kernel issues (roofline.issue).  Both come from one `ncu` capture of
the same kernel on a small case of the workload, scaled per pair.  This module turns
that capture into profiles/<kernel>_<workload>.json:

  python -m rkhs_ba_gb300.profiling <capture.ncu-rep> --kernel k_assoc_cta --pairs 2 \
      --command "<the ncu command that made the capture>" --out profiles/k_assoc_cta_global50k.json

It runs `ncu -i <capture> --page raw --csv` (no GPU needed) and averages the metrics
over the captured launches of the kernel.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
METRICS = ("dram__bytes_read.sum", "dram__bytes_write.sum", "smsp__inst_executed.sum", "gpu__time_duration.sum")


# unit strings of the raw page -> bytes or nanoseconds
_SCALE = {"byte": 1.0, "Kbyte": 1e3, "KB": 1e3, "Mbyte": 1e6, "MB": 1e6, "Gbyte": 1e9, "GB": 1e9,
          "nsecond": 1.0, "ns": 1.0, "usecond": 1e3, "us": 1e3, "msecond": 1e6, "ms": 1e6}


def _number(v: str) -> float:
    return float(v.replace(",", ""))


def read_capture(path: str, kernel: str) -> dict:
    """Mean of METRICS over the launches of `kernel` in the capture (values in the raw
    page's units: bytes, instructions, nanoseconds)."""
    out = subprocess.run(["ncu", "-i", path, "--page", "raw", "--csv"], check=True, capture_output=True,
                         text=True).stdout
    rows = list(csv.reader(io.StringIO(out)))
    head = rows[0]
    units = rows[1] if len(rows) > 1 else []
    col = {m: head.index(m) for m in METRICS if m in head}
    kcol = head.index("Kernel Name")
    acc = {m: [] for m in col}
    for r in rows[2:]:
        if len(r) <= kcol or kernel not in r[kcol]:
            continue
        for m, c in col.items():
            u = units[c] if c < len(units) else ""
            acc[m].append(_number(r[c]) * _SCALE.get(u, 1.0))
    return {m: sum(v) / len(v) for m, v in acc.items() if v}


def summarize(path: str, kernel: str, pairs: int, command: str) -> dict:
    m = read_capture(path, kernel)
    dram = m.get("dram__bytes_read.sum", 0.0) + m.get("dram__bytes_write.sum", 0.0)
    return {"kernel": kernel, "pairs_per_launch": pairs, "command": command,
            "dram_bytes_per_pair_launch": round(dram / pairs),
            "warp_instructions_per_pair_launch": round(m.get("smsp__inst_executed.sum", 0.0) / pairs),
            "gpu_time_ns_per_launch": round(m.get("gpu__time_duration.sum", 0.0)),
            "source": os.path.basename(path)}


def load(name: str) -> dict | None:
    """profiles/<name> as a dict, or None when absent."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        return json.load(fh)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("capture")
    ap.add_argument("--kernel", default="k_assoc_cta")
    ap.add_argument("--pairs", type=int, required=True)
    ap.add_argument("--command", required=True)
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    d = summarize(a.capture, a.kernel, a.pairs, a.command)
    with open(a.out, "w") as fh:
        json.dump(d, fh, indent=1)
        fh.write("\n")
    print(json.dumps(d))


if __name__ == "__main__":
    main()
