"""Summarise an ncu report (or a launch-list CSV) into the short text kept beside the benchmark.

    python -m mlgi.ncu_summary report.ncu-rep  > <kernel>_<workload>.md
    python -m mlgi.ncu_summary launches.csv    > launches_<workload>.md

A report summary ends each kernel with a `traffic[<kernel>] = <bytes>` line (DRAM read + write of
one launch) and an `issue[<kernel>] = <percent>` line (issue slots busy), which bench.py reads for
the roofline's `traffic` and `issue_busy_pct`.
"""
import collections
import csv
import io
import subprocess
import sys

METRICS = [
    ("gpu__time_duration.sum", "duration"),
    ("dram__bytes_read.sum", "DRAM read"),
    ("dram__bytes_write.sum", "DRAM write"),
    ("gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed", "DRAM throughput % of peak"),
    ("lts__throughput.avg.pct_of_peak_sustained_elapsed", "L2 throughput % of peak"),
    ("sm__throughput.avg.pct_of_peak_sustained_elapsed", "SM throughput % of peak"),
    ("smsp__issue_active.avg.pct_of_peak_sustained_active", "issue slots busy %"),
    ("sm__warps_active.avg.pct_of_peak_sustained_active", "warps active % (occupancy)"),
    ("smsp__inst_executed.sum", "warp instructions"),
    ("smsp__thread_inst_executed_per_inst_executed.ratio", "active threads per instruction"),
    ("sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active", "FMA pipe busy %"),
    ("sm__pipe_tensor_cycles_active.avg.pct_of_peak_sustained_active", "tensor pipe busy %"),
    ("launch__registers_per_thread", "registers per thread"),
    ("launch__occupancy_limit_shared_mem", "blocks/SM allowed by shared memory"),
]


_BYTES = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}


def _value(hdr, units, row, key, scale):
    """The metric's value in base units (scale maps its unit to a factor), or None if absent."""
    if key not in hdr or not row[hdr.index(key)]:
        return None
    u = units[hdr.index(key)]
    if u not in scale:
        return None
    return float(row[hdr.index(key)].replace(",", "")) * scale[u]


def report(path):
    out = subprocess.run(["ncu", "-i", path, "--page", "raw", "--csv"], stdout=subprocess.PIPE, text=True).stdout
    rows = list(csv.reader(io.StringIO(out)))
    hdr, units = rows[0], rows[1]
    for r in rows[2:]:
        name = r[hdr.index("Kernel Name")]
        print(f"## {name}\n")
        print("| metric | value |\n|---|---|")
        for key, label in METRICS:
            if key in hdr:
                print(f"| {label} (`{key}`) | {r[hdr.index(key)]} {units[hdr.index(key)]} |")
        # achieved rates of this launch: DRAM and L2 bytes, and L2 atomic/reduction requests, per second
        dur = _value(hdr, units, r, "gpu__time_duration.sum", {"nsecond": 1e-9, "ns": 1e-9, "usecond": 1e-6,
                                                                  "us": 1e-6, "msecond": 1e-3, "ms": 1e-3})
        if dur:
            dram = sum(_value(hdr, units, r, k, _BYTES) or 0.0 for k in ("dram__bytes_read.sum", "dram__bytes_write.sum"))
            print(f"| achieved DRAM GB/s (read + write / duration) | {dram / dur / 1e9:.1f} GB/s |")
            sectors = _value(hdr, units, r, "lts__t_sectors.sum", {"sector": 1.0, "": 1.0})
            if sectors is not None:
                print(f"| achieved L2 GB/s (`lts__t_sectors.sum` x 32 B / duration) | {sectors * 32 / dur / 1e9:.1f} GB/s |")
            atom = sum(_value(hdr, units, r, k, {"request": 1.0, "": 1.0}) or 0.0
                       for k in ("lts__t_requests_srcunit_tex_op_red.sum", "lts__t_requests_srcunit_tex_op_atom.sum"))
            if atom:
                print(f"| L2 atomic and reduction requests | {atom:.0f} ({atom / dur / 1e9:.1f} G/s) |")
        stalls = []
        for i, h in enumerate(hdr):
            if h.startswith("smsp__average_warps_issue_stalled") and h.endswith("per_issue_active.ratio") and r[i]:
                stalls.append((float(r[i].replace(",", "")), h[len("smsp__average_warps_issue_stalled_"):-len("_per_issue_active.ratio")]))
        stalls.sort(reverse=True)
        print("\nTop warp stall reasons (cycles per issued instruction): " +
              ", ".join(f"{n} {v:.2f}" for v, n in stalls[:6]) + "\n")
        rd = float(r[hdr.index("dram__bytes_read.sum")].replace(",", ""))
        wr = float(r[hdr.index("dram__bytes_write.sum")].replace(",", ""))
        scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
        rd *= scale.get(units[hdr.index("dram__bytes_read.sum")], 1)
        wr *= scale.get(units[hdr.index("dram__bytes_write.sum")], 1)
        short = name.split("(")[0].split("::")[-1].split("<")[0].replace("void ", "").strip()
        passes = {"vpl_process_kernel": "vpl_process", "ism_clear_kernel": "ism_clear", "ism_splat_kernel": "ism_splat",
                  "pull1_kernel": "pull1", "pullmid_kernel": "pullmid", "push1_kernel": "push1",
                  "push0_kernel": "push0", "fg_kernel": "final_gather"}
        print(f"traffic[{passes.get(short, short)}] = {rd + wr:.4e}  (DRAM read + write bytes of this launch)")
        issue = _value(hdr, units, r, "smsp__issue_active.avg.pct_of_peak_sustained_active", {"%": 1.0})
        if issue is not None:
            print(f"issue[{passes.get(short, short)}] = {issue:.1f}  (% of issue slots busy while a warp is resident)")
        print()


def launches(path):
    rows = list(csv.reader(open(path)))
    hdr, data = None, []
    for r in rows:
        if r and r[0] == "ID":
            hdr = r
            continue
        if hdr and len(r) == len(hdr):
            data.append(dict(zip(hdr, r)))
    agg = collections.OrderedDict()
    for d in data:
        if d.get("Metric Name") != "gpu__time_duration.sum":
            continue
        v = float(d["Metric Value"].replace(",", ""))
        v *= {"nsecond": 1e-3, "ns": 1e-3, "usecond": 1.0, "us": 1.0, "msecond": 1e3, "ms": 1e3}[d["Metric Unit"]]
        a = agg.setdefault(d["Kernel Name"].split("(")[0], [0, 0.0])
        a[0] += 1
        a[1] += v
    tot = sum(v[1] for v in agg.values())
    print("| kernel | launches | total us | share |\n|---|---|---|---|")
    for k, (n, t) in sorted(agg.items(), key=lambda x: -x[1][1]):
        print(f"| `{k}` | {n} | {t:.1f} | {100 * t / tot:.1f}% |")


if __name__ == "__main__":
    p = sys.argv[1]
    (report if p.endswith(".ncu-rep") else launches)(p)
