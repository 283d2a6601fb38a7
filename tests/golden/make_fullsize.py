"""Pins full-size generated databases to the oracle.

For every database spec, this script writes one row of a pin table:
  config, seed, scale, sha256 of the database written as txt, minsup,
  pattern count, sha256 of the oracle's output, max pattern edges (0 = none).
The output hash is over "<code>\\t<support>" lines in the reference's
traversal order with the sequential miner's label convention, each line
ending in a newline.

The oracle (oracle/_build/gspan_oracle, a C restatement of the reference's
src/gspan pinned to the reference binary on the golden runs) generates each
database itself (`gen` input) and mines it as root-subtree shares
(`--roots i/n`) in parallel on the host cores.  The reference's root loop
(src/gspan/gspan.cpp:300-351) shares nothing between root subtrees, so the
shares merged in root order are exactly the single-process output; the
k-th root group of share r is frequent root k*n + r.

Usage (from the repository root, after `make -C oracle`):
  python tests/golden/make_fullsize.py [--jobs N] [--parts P] SPEC...
  SPEC = config,seed,scale,minsup[,max_edges]    minsup: absolute, or a
         fraction of the graph count when it contains a '.'
  python tests/golden/make_fullsize.py --batch [--jobs N]
         the 64 databases of generator configuration 3 (seeds 1000-1063)
         at minsup 5%
  python tests/golden/make_fullsize.py --serving [--jobs N]
         one request per configuration-4 database (seeds 2000-2007): minsup
         1/2/5/10% in turn, max edges 4..8 in turn

Rows go to stdout.  The committed tables are fullsize.tsv (configurations 2,
4 and 5) and fullsize_batch.tsv (configuration 3).
"""
import argparse
import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
ORACLE = os.path.join(REPO, "oracle", "_build", "gspan_oracle")


def db_info(config, seed, scale):
    """sha256 of the generated database written as txt, and its graph count."""
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "db.txt")
        subprocess.check_call([ORACLE, "--write-gen", "%d,%d,%r" % (config, seed, scale), p])
        h = hashlib.sha256()
        n = 0
        with open(p, "rb") as f:
            for line in f:
                h.update(line)
                if line.startswith(b"t "):
                    n += 1
        return h.hexdigest(), n


def mine_share(config, seed, scale, minsup, max_edges, part, parts):
    cmd = [ORACLE, "gen", "%d,%d,%r" % (config, seed, scale), str(minsup)]
    if parts > 1:
        cmd += ["--roots", "%d/%d" % (part, parts)]
    if max_edges:
        cmd += ["--max-edges", str(max_edges)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle failed (%d): %s" % (r.returncode, r.stderr))
    return r.stdout.splitlines()


def root_groups(lines):
    """Split one share's output at its one-edge patterns (each frequent root
    is reported before its subtree)."""
    groups = []
    for line in lines:
        if ";" not in line.split("\t", 1)[0]:
            groups.append([])
        groups[-1].append(line)
    return groups


def merge(shares):
    gs = [root_groups(s) for s in shares]
    n = len(gs)
    out = []
    total = sum(len(g) for g in gs)
    for k in range(total):
        out.extend(gs[k % n][k // n])
    return out


def pin(specs, jobs, parts):
    """specs: (config, seed, scale, minsup or fraction, max_edges) -> rows"""
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        infos = list(ex.map(lambda s: db_info(s[0], s[1], s[2]), specs))
        resolved = []
        for s, (sha, n) in zip(specs, infos):
            ms = s[3]
            if isinstance(ms, float):
                ms = max(1, int(round(ms * n)))
            resolved.append((s[0], s[1], s[2], ms, s[4], sha, n))
        futs = {}
        for i, (c, seed, scale, ms, me, _, n) in enumerate(resolved):
            p = parts if n >= 100000 else 1
            for r in range(p):
                futs[(i, r)] = ex.submit(mine_share, c, seed, scale, ms, me, r, p)
        rows = []
        for i, (c, seed, scale, ms, me, sha, n) in enumerate(resolved):
            p = parts if n >= 100000 else 1
            lines = merge([futs[(i, r)].result() for r in range(p)]) if p > 1 else futs[(i, 0)].result()
            h = hashlib.sha256(("\n".join(lines) + "\n").encode()).hexdigest()
            rows.append("%d\t%d\t%r\t%s\t%d\t%d\t%s\t%d" % (c, seed, scale, sha, ms, len(lines), h, me))
            print(rows[-1], flush=True)
    return rows


def parse_spec(s):
    f = s.split(",")
    ms = float(f[3]) if "." in f[3] else int(f[3])
    return (int(f[0]), int(f[1]), float(f[2]), ms, int(f[4]) if len(f) > 4 else 0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--parts", type=int, default=24, help="root shares per database of 100,000 graphs or more")
    ap.add_argument("--batch", action="store_true")
    ap.add_argument("--serving", action="store_true")
    ap.add_argument("spec", nargs="*")
    a = ap.parse_args()
    if not os.path.exists(ORACLE):
        subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle")])
    specs = [parse_spec(s) for s in a.spec]
    if a.batch:
        specs += [(3, 1000 + i, 1.0, 0.05, 0) for i in range(64)]
    if a.serving:
        specs += [(4, 2000 + i, 1.0, [0.01, 0.02, 0.05, 0.10][i % 4], 4 + i % 5) for i in range(8)]
    if not specs:
        ap.error("no databases given")
    pin(specs, a.jobs, a.parts)


if __name__ == "__main__":
    sys.exit(main())
