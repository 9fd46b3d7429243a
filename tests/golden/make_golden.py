"""Generate the golden fixtures that pin the oracle to the reference.

Each fixture is a small seeded graph plus a raw (untidied) batch, run through
the reference's own CPU code (oracle/ref_harness.cpp compiled against the
headers of puzzlef/pagerank-cuda-dynamic by `make -C oracle ref`).  The
fixture stores the inputs and what the reference produced:

  x_off/x_edg, xt_off/xt_edg/xt_dat     csrCreate*W of x and its transpose
  del_u/del_v, ins_u/ins_v              tidyBatchUpdateU output (batch.hxx:200)
  y_off/y_edg, yt_off/yt_edg/yt_dat     after applyBatchUpdateOmpU + transpose
  df_flags, dt_flags                    pagerankAffectedFrontierW / ...TraversalW
  static_x_*, static_y_*                pagerankStaticOmp (pagerank.hxx:474)
  nd_y_*                                pagerankNaiveDynamic<false> from static_x
  exact_y_ranks                         pagerankStaticOmp with tol 1e-100

Run from the repository root where the reference headers exist:
    make -C oracle ref REF_INC=<reference>/inc && python tests/golden/make_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def rmat_edges(scale, ef, rng, a=0.57, b=0.19, c=0.19):
    n = 1 << scale
    m = ef * n
    u = np.zeros(m, np.int64)
    v = np.zeros(m, np.int64)
    for _ in range(scale):
        p = rng.random(m)
        ub = (p >= a + b).astype(np.int64)
        vb = (((p >= a) & (p < a + b)) | (p >= a + b + c)).astype(np.int64)
        u = (u << 1) | ub
        v = (v << 1) | vb
    return n, u, v


def grid_edges(w, rng, frac=0.05):
    n = w * w
    us, vs = [], []
    r, c = np.divmod(np.arange(n), w)
    for dr, dc in ((0, 1), (0, -1), (1, 0), (-1, 0)):
        ok = (r + dr >= 0) & (r + dr < w) & (c + dc >= 0) & (c + dc < w)
        us.append(np.arange(n)[ok])
        vs.append(((r + dr) * w + (c + dc))[ok])
    pick = rng.random(n) < frac
    d = rng.integers(0, 4, n)
    dr = np.where(d < 2, -1, 1)
    dc = np.where(d % 2 == 0, -1, 1)
    ok = pick & (r + dr >= 0) & (r + dr < w) & (c + dc >= 0) & (c + dc < w)
    s = np.arange(n)[ok]
    t = ((r + dr) * w + (c + dc))[ok]
    us += [s, t]
    vs += [t, s]
    return n, np.concatenate(us), np.concatenate(vs)


def hub_edges(n, rng):
    # vertex 0 receives an edge from everyone (in-degree n), vertex 1 from
    # every third vertex, plus a sprinkle of random edges
    u = [np.arange(1, n), np.arange(2, n, 3), rng.integers(0, n, 4 * n)]
    v = [np.zeros(n - 1, np.int64), np.ones(len(range(2, n, 3)), np.int64), rng.integers(0, n, 4 * n)]
    return n, np.concatenate(u), np.concatenate(v)


def web_edges(n, rng, window=64):
    deg = np.minimum(1000, np.floor(2.0 * rng.random(n) ** (-1 / 1.1))).astype(np.int64)
    u = np.repeat(np.arange(n), deg)
    local = rng.random(len(u)) < 0.7
    off = rng.integers(-window, window + 1, len(u))
    v = np.where(local, np.clip(u + off, 0, n - 1), rng.integers(0, n, len(u)))
    return n, u, v


def with_self_loops(n, u, v):
    u = np.concatenate([u, np.arange(n)])
    v = np.concatenate([v, np.arange(n)])
    key = np.unique(u.astype(np.int64) * n + v)
    return key // n, key % n


def random_batch(n, u, v, size, rng, ins_frac=0.8, extra_noise=True):
    ni = int(round(size * ins_frac))
    nd = size - ni
    iu = rng.integers(0, n, ni)
    iv = rng.integers(0, n, ni)
    nonself = np.nonzero(u != v)[0]
    pick = rng.choice(nonself, size=min(nd, len(nonself)), replace=False) if nd else np.zeros(0, np.int64)
    du, dv = u[pick], v[pick]
    if extra_noise and size:
        # exercise tidyBatchUpdateU: duplicates, existing insertions,
        # missing deletions
        k = max(1, size // 10)
        iu = np.concatenate([iu, iu[:k], u[:k]])
        iv = np.concatenate([iv, iv[:k], v[:k]])
        du = np.concatenate([du, du[:k], rng.integers(0, n, k)])
        dv = np.concatenate([dv, dv[:k], rng.integers(0, n, k)])
    return du, dv, iu, iv


def run_harness(n, u, v, du, dv, iu, iv, tol):
    lines = [f"{n} {len(u)} {tol!r}"]
    lines += [f"{a} {b}" for a, b in zip(u.tolist(), v.tolist())]
    lines.append(str(len(du)))
    lines += [f"{a} {b}" for a, b in zip(du.tolist(), dv.tolist())]
    lines.append(str(len(iu)))
    lines += [f"{a} {b}" for a, b in zip(iu.tolist(), iv.tolist())]
    env = dict(os.environ, OMP_NUM_THREADS="4")
    out = subprocess.run([HARNESS], input="\n".join(lines) + "\n", capture_output=True,
                         text=True, check=True, env=env).stdout.split("\n")
    rec, i = {}, 0
    while i < len(out):
        if not out[i].strip():
            i += 1
            continue
        name, kind, cnt = out[i].split()
        cnt = int(cnt)
        vals = out[i + 1].split() if cnt else []
        if kind == "u":
            rec[name] = np.array([int(x) for x in vals], dtype=np.int64)
        else:
            rec[name] = np.array([float.fromhex(x) for x in vals], dtype=np.float64)
        i += 2
    return rec


def make_case(name, n, u, v, batch, tol=1e-10):
    u, v = with_self_loops(n, np.asarray(u, np.int64), np.asarray(v, np.int64))
    du, dv, iu, iv = batch(n, u, v)
    rec = run_harness(n, u, v, du, dv, iu, iv, tol)
    rec.update(n=np.int64(n), tol=np.float64(tol),
               raw_del_u=du, raw_del_v=dv, raw_ins_u=iu, raw_ins_v=iv)
    for k in ("x_off", "x_edg", "xt_off", "xt_edg", "xt_dat", "del_u", "del_v", "ins_u",
              "ins_v", "y_off", "y_edg", "yt_off", "yt_edg", "yt_dat", "df_flags", "dt_flags",
              "raw_del_u", "raw_del_v", "raw_ins_u", "raw_ins_v"):
        rec[k] = rec[k].astype(np.uint32)
    for k in ("static_x_iters", "static_y_iters", "nd_y_iters"):
        rec[k] = np.int64(rec[k][0])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print(f"{name}: n={n} m={len(u)} del={len(rec['del_u'])} ins={len(rec['ins_u'])} "
          f"iters x={rec['static_x_iters']} y={rec['static_y_iters']} nd={rec['nd_y_iters']} "
          f"df={int(rec['df_flags'].sum())} dt={int(rec['dt_flags'].sum())}")


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: make -C oracle ref REF_INC=<reference>/inc")
    rng = np.random.default_rng(42)
    frac = lambda f: (lambda n, u, v: random_batch(n, u, v, max(1, int(f * len(u))), rng))
    n, u, v = rmat_edges(8, 16, rng)
    make_case("rmat8", n, u, v, frac(1e-2))
    n, u, v = rmat_edges(10, 16, rng)
    make_case("rmat10", n, u, v, frac(1e-3))
    n, u, v = rmat_edges(12, 16, rng)
    make_case("rmat12", n, u, v, frac(1e-4))
    n, u, v = grid_edges(24, rng)
    make_case("grid24", n, u, v, frac(2e-3))
    n, u, v = hub_edges(3000, rng)
    make_case("hub3000", n, u, v, frac(1e-3))
    n, u, v = web_edges(4000, rng)
    make_case("web4000", n, u, v, frac(1e-3))
    # edge cases: single vertex, empty batch, deletions only, insertions only
    make_case("single", 1, [], [], lambda n, u, v: (np.zeros(0, np.int64),) * 4)
    n, u, v = rmat_edges(7, 8, rng)
    make_case("rmat7_empty_batch", n, u, v, lambda n, u, v: (np.zeros(0, np.int64),) * 4)
    make_case("rmat7_del_only", n, u, v,
              lambda n, u, v: random_batch(n, u, v, 30, rng, ins_frac=0.0, extra_noise=False))
    make_case("rmat7_ins_only", n, u, v,
              lambda n, u, v: random_batch(n, u, v, 30, rng, ins_frac=1.0, extra_noise=False))


if __name__ == "__main__":
    main()
