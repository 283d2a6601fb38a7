"""Edge cases against the oracle: deep patterns (long frequent paths: the
count kernel's 32- and 64-column variants and the host canonicality check
beyond 32 vertices), highly symmetric graphs (complete graphs with one label:
many automorphisms and backward edges), graphs without edges, and supports
where nothing is frequent.  Both extension strategies."""
import random

import pytest

from conftest import run_oracle, to_lines

pytestmark = pytest.mark.gpu


def _write(path, graphs):
    lines = []
    for gi, (vl, edges) in enumerate(graphs):
        lines.append("t # %d" % gi)
        lines += ["v %d %d" % (v, l) for v, l in enumerate(vl)]
        lines += ["e %d %d %d" % (a, b, l) for a, b, l in edges]
    path.write_text("\n".join(lines) + "\n")
    return str(path)


def _check(gs, oracle, path, minsup, extra=(), **kw):
    want = run_oracle(oracle, "txt", path, minsup, list(extra))
    db = gs.Database.load(path, "txt")
    me = {"max_edges": int(extra[1])} if extra else {}
    for ext in ("rmpath", "lists"):
        pats, stats = gs.mine(db, minsup, label_style=gs.LABELS_SEQ, extension=ext, **me, **kw)
        assert to_lines(pats, gs) == want, ext
    return want, stats


def test_deep_paths(gs, oracle, tmp_path):
    # 12 graphs sharing one labelled path of 44 vertices, each with its own
    # chords: every shared sub-path is frequent, up to 43 edges (44 vertices)
    r = random.Random(3)
    graphs = []
    for gi in range(12):
        n = 44
        vl = [v % 3 for v in range(n)]
        edges = [(v, v + 1, 0) for v in range(n - 1)]
        have = {(v, v + 1) for v in range(n - 1)}
        while len(edges) < n + 1:
            a, b = sorted(r.sample(range(n), 2))
            if b - a > 1 and (a, b) not in have:
                have.add((a, b))
                edges.append((a, b, 1 + gi % 2))
        graphs.append((vl, edges))
    want, stats = _check(gs, oracle, _write(tmp_path / "paths.txt", graphs), 10)
    assert max(line.count("(") for line in want) >= 40
    assert stats["min_host_checks"] > 0   # patterns beyond 32 vertices are checked on the host


@pytest.mark.parametrize("n,labels", [(6, 1), (6, 2), (5, 3)])
def test_complete_graphs(gs, oracle, tmp_path, n, labels):
    # complete graphs: every connected subgraph frequent, many automorphisms
    r = random.Random(n * 10 + labels)
    graphs = []
    for gi in range(10):
        vl = [r.randrange(labels) if gi % 3 else v % labels for v in range(n)]
        edges = [(a, b, 0) for a in range(n) for b in range(a + 1, n)]
        graphs.append((vl, edges))
    _check(gs, oracle, _write(tmp_path / "complete.txt", graphs), 4)


def test_graphs_without_edges_and_nothing_frequent(gs, oracle, tmp_path):
    # isolated vertices contribute no patterns; at a high support nothing is
    # frequent and the output is empty
    r = random.Random(11)
    graphs = []
    for gi in range(20):
        n = r.randint(1, 8)
        vl = [r.randrange(4) for _ in range(n)]
        edges = []
        if gi % 4 and n > 1:
            for v in range(1, n):
                edges.append((r.randrange(v), v, r.randrange(2)))
        graphs.append((vl, edges))
    path = _write(tmp_path / "sparse.txt", graphs)
    want, _ = _check(gs, oracle, path, 3)
    assert want
    empty, _ = _check(gs, oracle, path, 19)
    assert empty == []


def _paths(n, count, seed):
    r = random.Random(seed)
    graphs = []
    for gi in range(count):
        vl = [v % 3 for v in range(n)]
        edges = [(v, v + 1, 0) for v in range(n - 1)]
        # a chord of a graph-specific label: not frequent
        a = r.randrange(n - 2)
        edges.append((a, a + 2, 5 + gi))
        graphs.append((vl, edges))
    return graphs


def test_paths_at_the_vertex_limit(gs, oracle, tmp_path):
    # 64-vertex paths: frequent sub-paths up to 63 edges and 64 vertices, the
    # largest patterns the miner takes (bit-set membership, 64-column kernels)
    want, _ = _check(gs, oracle, _write(tmp_path / "p64.txt", _paths(64, 12, 1)), 10)
    assert max(line.count("(") for line in want) == 63


def test_paths_beyond_the_vertex_limit(gs, oracle, tmp_path):
    # 70-vertex paths (the general membership path): patterns of more than 64
    # vertices are refused with GS_ERR_LIMIT, never cut short silently; with
    # max_edges they are mined exactly
    path = _write(tmp_path / "p70.txt", _paths(70, 12, 2))
    db = gs.Database.load(path, "txt")
    with pytest.raises(gs.GSpanError) as e:
        gs.mine(db, 10)
    assert e.value.status == 8  # GS_ERR_LIMIT
    _check(gs, oracle, path, 10, ["--max-edges", "60"])


def test_many_labels(gs, oracle, tmp_path):
    # 3,000 vertex labels and 40 edge labels: large label alphabets and pair
    # tables, most roots infrequent
    r = random.Random(21)
    graphs = []
    for gi in range(100):
        n = r.randint(8, 20)
        vl = [6 + r.randrange(3000) if r.random() < 0.3 else r.randrange(3) for _ in range(n)]
        edges = [(r.randrange(v), v, 2 + r.randrange(40) if r.random() < 0.2 else r.randrange(2)) for v in range(1, n)]
        graphs.append((vl, edges))
    want, _ = _check(gs, oracle, _write(tmp_path / "labels.txt", graphs), 5)
    assert len(want) > 50 and max(line.count("(") for line in want) >= 3


def test_high_degree_stars(gs, oracle, tmp_path):
    # star graphs of degree 20: rows with hundreds of items, over a million
    # embeddings, the record buffer outgrown on a fresh engine
    graphs = []
    for gi in range(10):
        n = 21 + gi % 3
        vl = [0] + [1 + (v % 2 if gi % 2 else 0) for v in range(1, n)]
        edges = [(0, v, 0) for v in range(1, n)]
        graphs.append((vl, edges))
    gs.engine_reset()
    _check(gs, oracle, _write(tmp_path / "stars.txt", graphs), 8, ["--max-edges", "4"])


@pytest.mark.parametrize("name", ["fixture_get_test_database.txt", "fixture_get_labeled_test_database.txt",
                                  "fixture_get_labeled_test_database2.txt"])
def test_minsup_one(gs, oracle, name):
    # support 1: every connected subgraph of every graph is frequent
    import os
    from conftest import GOLDEN
    _check(gs, oracle, os.path.join(GOLDEN, name), 1)


def test_more_partitions_than_roots(gs):
    # root shares beyond the number of frequent roots are empty, and the
    # shares still merge into the single-process output
    import os
    from conftest import GOLDEN
    from gpu_graph_mining_gb300.partition import merge_root_partitions
    db = gs.Database.load(os.path.join(GOLDEN, "fixture_get_labeled_test_database.txt"), "txt")
    want, _ = gs.mine_collect(db, 3)
    roots = sum(1 for code, _ in want if len(code) == 1)
    n = roots + 5
    parts = [gs.mine_collect(db, 3, root_part=r, root_parts=n)[0] for r in range(n)]
    assert sum(1 for p in parts if not p) >= 5
    assert merge_root_partitions(parts) == want


@pytest.mark.parametrize("device", [False, True])
def test_empty_and_degenerate_arrays(gs, device):
    # no graphs, and graphs of one vertex without edges: both ingest paths
    # accept them, and mining refuses a support it cannot reach (never a crash)
    empty = gs.Database.from_arrays(0, 0, [], [], [], [0], 0, device=device)
    assert len(empty) == 0
    with pytest.raises(gs.GSpanError) as e:
        gs.mine(empty, 1)
    assert e.value.status == 6  # GS_ERR_MINSUP_TOO_LARGE
    # three graphs of one vertex each (max 1 vertex per graph, no edges)
    single = gs.Database.from_arrays(3, 1, [], [], [4, 4, 7], [0, 0, 0, 0], 3, device=device)
    assert len(single) == 3
    pats, _ = gs.mine(single, 2)
    assert pats == []


@pytest.mark.parametrize("ft,dbf,minsup,out", [
    ("txt", "cfg1_seed1.txt", 10, "out_cfg1_seed1_s10.txt"),
    ("bin", "fixture_labeled.bin", 2, "out_fixture_labeled_s2.txt"),
    ("txt", "fixture_get_labeled_test_database2.txt", 3, "out_fixture_get_labeled_test_database2_s3.txt"),
])
def test_cli_output_is_golden(gs, tmp_path, ft, dbf, minsup, out):
    # the command-line miner (the reference mains' interface) prints the
    # golden patterns, in order, to stdout or to a file ("-": count only),
    # and the reference's count line on stderr
    import os
    import subprocess
    from conftest import GOLDEN, read_lines
    want = read_lines(os.path.join(GOLDEN, out))
    cmd = [gs.CLI_PATH, ft, os.path.join(GOLDEN, dbf), str(minsup)]
    r = subprocess.run(cmd + ["--seq-labels"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == want
    assert "total_frequent_graphs=%d" % len(want) in r.stderr
    path = str(tmp_path / "patterns.txt")
    r = subprocess.run(cmd + [path, "--seq-labels"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout == ""
    assert read_lines(path) == want
    r = subprocess.run(cmd + ["-"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout == ""
    assert "total_frequent_graphs=%d" % len(want) in r.stderr
