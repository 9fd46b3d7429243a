"""Result lines in the reference driver's log format, and their parsing.

glog_line() writes the line main.cu:54-61 prints for every technique and
batch; parse_log() reads a log of such lines (ours or the reference's) into
rows, and write_csv() / write_csv_dir() / write_json() store them -- what the
reference's process.js does, with its result pattern brought up to the line
main.cu prints today (the "batchi" field and the init / mark / comp times
that process.js's pattern predates).
"""
import csv
import ctypes as C
import json
import os
import re

from ._lib import Result, check, load

GLOG = re.compile(
    r"^\{-(?P<deletions_fraction>\S+?)/\+(?P<insertions_fraction>\S+?) batchf, (?P<batch_index>\d+) batchi, "
    r"(?P<max_threads>\d+) threads\} -> \{\s*(?P<time>\S+?)ms,\s*(?P<initialization_time>\S+?)ms init,\s*"
    r"(?P<marking_time>\S+?)ms mark,\s*(?P<computation_time>\S+?)ms comp,\s*(?P<iterations>\d+) iter,\s*"
    r"(?P<error>\S+?) err\} (?P<technique>\w+)")
# the older pattern of process.js (no batch index, one time)
GLOG_OLD = re.compile(r"^\{-(?P<deletions_fraction>.+?)/\+(?P<insertions_fraction>.+?) batchf, (?P<max_threads>.+?) "
                      r"threads\} -> \{(?P<time>.+?)ms, (?P<iterations>.+?) iter, (?P<error>.+?) err\} (?P<technique>\w+)")
OMP = re.compile(r"^OMP_NUM_THREADS=(\d+)")
GRAPH = re.compile(r"^Loading graph (?:.*/)?(.+?)\.\w+ \.\.\.")
ORDER = re.compile(r"^order: (\d+) size: (\d+) \[directed\] \{\}")
STAMP = re.compile(r"^\d+-\d+-\d+ \d+:\d+:\d+\s+")
NUMERIC = ("deletions_fraction", "insertions_fraction", "batch_index", "max_threads", "time",
           "initialization_time", "marking_time", "computation_time", "iterations", "error")


def glog_line(result, technique, err, batch_index=0, threads=0, deletions_fraction=0.0, insertions_fraction=0.0):
    """The main.cu:56-59 line (no newline) for a result dict (or prx_result)."""
    r = result if isinstance(result, Result) else Result(**{k: result[k] for k in (
        "iterations", "time_ms", "initialization_time_ms", "marking_time_ms", "computation_time_ms")})
    buf = C.create_string_buffer(512)
    n = load().prx_format_glog(buf, len(buf), float(deletions_fraction), float(insertions_fraction),
                               int(batch_index), int(threads), C.byref(r), float(err), technique.encode())
    if n < 0:
        check(-n, "prx_format_glog")
    return buf.value.decode()


def parse_log(text):
    """Rows (dicts) of every result line, each with the graph, thread count,
    order and size in force where it appears (process.js readLog)."""
    rows, state = [], {}
    for ln in text.replace("\r\n", "\n").split("\n"):
        ln = STAMP.sub("", ln)
        m = OMP.match(ln)
        if m:
            state["omp_num_threads"] = float(m.group(1))
            continue
        m = GRAPH.match(ln)
        if m:
            state["graph"] = m.group(1)
            continue
        m = ORDER.match(ln)
        if m:
            state["order"], state["size"] = float(m.group(1)), float(m.group(2))
            continue
        m = GLOG.match(ln) or GLOG_OLD.match(ln)
        if m:
            row = dict(state)
            for k, v in m.groupdict().items():
                row[k] = float(v) if k in NUMERIC else v
            rows.append(row)
    return rows


def write_csv(path, rows):
    """All rows in one CSV (process.js `csv`); values quoted as there."""
    cols = list(rows[0].keys()) if rows else []
    for r in rows:
        for k in r:
            if k not in cols:
                cols.append(k)
    with open(path, "w", newline="") as f:
        w = csv.writer(f, quoting=csv.QUOTE_ALL)
        w.writerow(cols)
        for r in rows:
            w.writerow([r.get(k, "") for k in cols])


def write_csv_dir(path, rows):
    """One CSV per graph (process.js `csv-dir`)."""
    os.makedirs(path, exist_ok=True)
    by = {}
    for r in rows:
        by.setdefault(r.get("graph", "graph"), []).append(r)
    for g, rs in by.items():
        write_csv(os.path.join(path, g + ".csv"), rs)


def write_json(path, rows):
    with open(path, "w") as f:
        json.dump(rows, f, indent=1)


def main(argv=None):
    """python -m pagerank_gb300.report csv|json <log> <out>  (csv to a
    directory when <out> has no extension, as process.js does)."""
    import sys
    cmd, log, out = (argv or sys.argv[1:])[:3]
    with open(log) as f:
        rows = parse_log(f.read())
    if cmd == "csv":
        (write_csv_dir if os.path.splitext(out)[1] == "" else write_csv)(out, rows)
    elif cmd == "json":
        write_json(out, rows)
    else:
        raise SystemExit(f'error: "{cmd}"?')


if __name__ == "__main__":
    main()
