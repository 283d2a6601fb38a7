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
