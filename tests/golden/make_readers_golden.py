"""Generate the golden fixtures of the edge-list readers and the graph ingest.

Writes small input files under tests/golden/readers/ (seeded SNAP temporal
text, MatrixMarket files, and a hand-written file of edge cases), runs the
reference's own readers and graph builder on them (oracle/ref_readers.cpp,
compiled against the headers of puzzlef/pagerank-cuda-dynamic by
`make -C oracle ref`), and stores what they produced in readers.npz:

  pieces_<file>_u<i>/_v<i>    readTemporalDo (inc/snap.hxx:41-52) per piece
  mtx_<file>_header/_u/_v     readMtxDo (inc/mtx.hxx:119-135), 1-based ids
  pipe_*                      main.cu's graph flow (x, xt, then per batch
                              raw and tidied insertions, y, yt; each y is
                              the next batch's x), 0-based CSRs

Run from the repository root where the reference headers exist:
    make -C oracle ref REF_INC=<reference>/inc && python tests/golden/make_readers_golden.py
"""
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "readers")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_readers")

# (file, rows, piece sizes) for the piecewise reads
PIECES = [
    ("temporal_small.txt", 500, [1000, 2000, 0, 3000, 500]),
    ("temporal_edge.txt", 12, [3, 2, 4, 100, 5]),
]
MTX = ["general.mtx", "symmetric.mtx", "skew.mtx", "rect.mtx", "array.mtx", "crlf.mtx"]
# main.cu's flow: file, rows, size (lines), batch fraction, batches
PIPELINE = ("temporal_small.txt", 500, 6000, 0.01, 3)


def write_inputs():
    os.makedirs(OUT, exist_ok=True)
    rng = np.random.default_rng(2024)
    # temporal: 6000 lines "u v t", ids 1..500 with a skew towards low ids,
    # duplicates and some self-loops, timestamps ascending
    n, m = 500, 6000
    u = np.minimum((rng.pareto(1.2, m) * 20).astype(np.int64), n - 1) + 1
    v = np.where(rng.random(m) < 0.02, u, rng.integers(1, n + 1, m))
    dup = rng.random(m) < 0.05
    v[1:][dup[1:]] = v[:-1][dup[1:]]
    u[1:][dup[1:]] = u[:-1][dup[1:]]
    t = np.cumsum(rng.integers(0, 50, m)) + 1_200_000_000
    with open(os.path.join(OUT, "temporal_small.txt"), "w") as f:
        f.write("".join(f"{a} {b} {c}\n" for a, b, c in zip(u.tolist(), v.tolist(), t.tolist())))
    # hand-written edge cases: tabs, leading blanks, CRLF, leading zeros,
    # a third column, a line with one number, a line with text after the
    # first number, an empty line, and a last line without a newline
    edge = ("1 2\n"
            "\t3\t4\n"
            "  5 6 99\r\n"
            "007 8\n"
            "9\n"              # one number: ends the first-but-one piece
            "10 11\n"
            "12 1 x\n"
            "2abc 3\n"         # text after the first number: ends a piece
            "4 5\n"
            "\n"               # empty line: ends a piece
            "6 7\n"
            "8 9\n"
            "11 12")           # no newline at the end
    with open(os.path.join(OUT, "temporal_edge.txt"), "w", newline="") as f:
        f.write(edge)
    files = {
        "general.mtx": ("%%MatrixMarket matrix coordinate pattern general\n"
                        "% a comment line\n"
                        "%\n"
                        "6 6 9\n"
                        "1 2\n2 3\n3 1\n4 4\n5 6\n6 5\n1 2\n2 1\n3 6\n"),
        "symmetric.mtx": ("%%MatrixMarket matrix coordinate real symmetric\n"
                          "% entries of the lower triangle, with values\n"
                          "5 5 7\n"
                          "1 1 1.0\n2 1 0.5\n3 1 2.0\n4 3 1.5\n5 5 3.0\n5 2 0.25\n4 4 1.0\n"),
        "skew.mtx": ("%%MatrixMarket matrix coordinate real skew-symmetric\n"
                     "4 4 3\n"
                     "2 1 1.0\n3 2 -1.0\n4 1 2.0\n"),
        "rect.mtx": ("%%MatrixMarket matrix coordinate integer general\n"
                     "5 8 6\n"
                     "1 8 1\n2 7 1\n5 1 1\n3 3 1\n4 6 1\n5 8 1\n"),
        "array.mtx": ("%%MatrixMarket matrix array real general\n"
                      "2 2\n"
                      "1.0\n2.0\n3.0\n4.0\n"),
        "crlf.mtx": ("%%MatrixMarket matrix coordinate pattern symmetric\r\n"
                     "%comment\r\n"
                     "4 4 4\r\n"
                     "2 1\r\n3 1\r\n4 2\r\n4 3"),
    }
    for name, text in files.items():
        with open(os.path.join(OUT, name), "w", newline="") as f:
            f.write(text)


def run(args):
    env = dict(os.environ, OMP_NUM_THREADS="4")
    out = subprocess.run([HARNESS, *map(str, args)], capture_output=True, text=True, check=True,
                         env=env).stdout.split("\n")
    rec, i = {}, 0
    while i < len(out):
        if not out[i].strip():
            i += 1
            continue
        name, kind, cnt = out[i].split()
        cnt = int(cnt)
        vals = out[i + 1].split() if cnt else []
        rec[name] = np.array([int(x) for x in vals], dtype=np.int64)
        i += 2
    return rec


def main():
    write_inputs()
    fx = {}
    for name, rows, sizes in PIECES:
        rec = run(["pieces", os.path.join(OUT, name), rows, *sizes])
        stem = name.split(".")[0]
        fx[f"pieces_{stem}_rows"] = np.int64(rows)
        fx[f"pieces_{stem}_sizes"] = np.array(sizes, np.int64)
        for k, a in rec.items():
            fx[f"pieces_{stem}_{k}"] = a
    for name in MTX:
        rec = run(["mtx", os.path.join(OUT, name)])
        stem = name.split(".")[0]
        for k, a in rec.items():
            fx[f"mtx_{stem}_{k}"] = a
    name, rows, size, frac, batches = PIPELINE
    rec = run(["pipeline", os.path.join(OUT, name), rows, size, frac, batches])
    fx["pipe_rows"], fx["pipe_size"] = np.int64(rows), np.int64(size)
    fx["pipe_frac"], fx["pipe_batches"] = np.float64(frac), np.int64(batches)
    for k, a in rec.items():
        fx[f"pipe_{k}"] = a
    np.savez_compressed(os.path.join(OUT, "readers.npz"), **fx)
    print(f"wrote {len(fx)} arrays to {os.path.join(OUT, 'readers.npz')}")


if __name__ == "__main__":
    main()
