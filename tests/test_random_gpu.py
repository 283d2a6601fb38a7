"""Randomised differential tests against the oracle: seeded random databases
(trees with extra edges for cycles, 1-6 vertex labels and 1-4 edge labels,
graphs of 2-24 or 66-90 vertices, supports of 10-50%, with or without an
edge cap), mined with both extension strategies.  Every case must match the
oracle line for line."""
import random

import pytest

from conftest import run_oracle, to_lines

pytestmark = pytest.mark.gpu


def _case(seed):
    r = random.Random(seed)
    ng = r.randint(5, 40)
    vl_n = r.choice([1, 2, 3, 4, 6])
    el_n = r.choice([1, 2, 3, 4])
    big = r.random() < 0.15         # graphs beyond 64 vertices: the general membership path
    dense = r.choice([0.0, 0.1, 0.3, 0.6])
    graphs = []
    for _ in range(ng):
        n = r.randint(66, 90) if big else r.randint(2, 24)
        vl = [r.randrange(vl_n) for _ in range(n)]
        edges = {}
        for v in range(1, n):
            edges[(r.randrange(v), v)] = r.randrange(el_n)
        for _ in range(int(dense * n)):
            a, b = sorted(r.sample(range(n), 2))
            edges.setdefault((a, b), r.randrange(el_n))
        graphs.append((vl, [(a, b, l) for (a, b), l in sorted(edges.items())]))
    minsup = min(ng - 1, max(1, int(ng * r.choice([0.1, 0.2, 0.3, 0.5]))))
    max_edges = r.choice([3, 4]) if big else r.choice([0, 3, 4, 5, 6])
    if dense >= 0.3 and max_edges == 0:
        max_edges = 5
    return graphs, minsup, max_edges


def _write(path, graphs):
    lines = []
    for gi, (vl, edges) in enumerate(graphs):
        lines.append("t # %d" % gi)
        lines += ["v %d %d" % (v, l) for v, l in enumerate(vl)]
        lines += ["e %d %d %d" % (a, b, l) for a, b, l in edges]
    path.write_text("\n".join(lines) + "\n")
    return str(path)


@pytest.mark.parametrize("group", range(8))
def test_random_databases_vs_oracle(gs, oracle, tmp_path, group):
    for seed in range(group * 50, group * 50 + 50):
        graphs, minsup, max_edges = _case(seed)
        path = _write(tmp_path / ("case%d.txt" % seed), graphs)
        extra = ["--max-edges", str(max_edges)] if max_edges else []
        want = run_oracle(oracle, "txt", path, minsup, extra)
        db = gs.Database.load(path, "txt")
        for ext in ("rmpath", "lists"):
            pats, _ = gs.mine(db, minsup, max_edges=max_edges, label_style=gs.LABELS_SEQ, extension=ext)
            assert to_lines(pats, gs) == want, (seed, ext, minsup, max_edges)
        db.free()


@pytest.mark.parametrize("group", range(4))
def test_random_batches_vs_oracle(gs, oracle, tmp_path, group):
    # ten random databases (different label alphabets, graph sizes and
    # supports) mined together in shared waves, each against the oracle
    seeds = range(1000 + group * 10, 1000 + group * 10 + 10)
    cases = [_case(seed) for seed in seeds]
    # one edge cap per batch: the largest of the cases' caps, 5 where a case has none
    cap = max(me if me else 5 for _, _, me in cases)
    dbs, sups, wants = [], [], []
    for seed, (graphs, minsup, _) in zip(seeds, cases):
        path = _write(tmp_path / ("batch%d.txt" % seed), graphs)
        wants.append(run_oracle(oracle, "txt", path, minsup, ["--max-edges", str(cap)]))
        dbs.append(gs.Database.load(path, "txt"))
        sups.append(minsup)
    for ext in ("rmpath", "lists"):
        got, _ = gs.mine_batch(dbs, sups, max_edges=cap, label_style=gs.LABELS_SEQ, extension=ext)
        for seed, g, w in zip(seeds, got, wants):
            assert to_lines(g, gs) == w, (seed, ext)


def test_random_device_ingest(gs, tmp_path):
    # random databases through the reference's cudabin arrays and the device
    # ingest mine exactly as the same databases read from text
    import numpy as np
    for seed in range(2000, 2040):
        graphs, minsup, max_edges = _case(seed)
        path = _write(tmp_path / ("ing%d.txt" % seed), graphs)
        host = gs.Database.load(path, "txt")
        cb = str(tmp_path / ("ing%d.cudabin" % seed))
        host.write(cb, "cudabin")
        raw = np.fromfile(cb, dtype=np.int32)
        n, esz, maxv, vc = (int(x) for x in raw[:4])
        o = 4
        edges = raw[o:o + esz]; o += esz
        elab = raw[o:o + esz]; o += esz
        vlab = raw[o:o + n * maxv]; o += n * maxv
        voff = raw[o:o + n * maxv + 1]
        dev = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc, device=True)
        want, _ = gs.mine_collect(host, minsup, max_edges=max_edges)
        got, _ = gs.mine_collect(dev, minsup, max_edges=max_edges)
        assert got == want, seed
        host.free()
        dev.free()


def test_concurrent_callers(gs, tmp_path):
    # host threads calling the library at once: device ingests, mining of
    # resident and of freshly ingested databases, both strategies, frees;
    # every result equals the same call made alone
    import threading
    import numpy as np
    cases = [_case(seed) for seed in range(3000, 3008)]
    paths = [_write(tmp_path / ("cc%d.txt" % i), g) for i, (g, _, _) in enumerate(cases)]
    dbs = [gs.Database.load(p, "txt") for p in paths]
    arrays = []
    for i, db in enumerate(dbs):
        cb = str(tmp_path / ("cc%d.cudabin" % i))
        db.write(cb, "cudabin")
        raw = np.fromfile(cb, dtype=np.int32)
        n, esz, maxv, vc = (int(x) for x in raw[:4])
        o = 4
        parts = []
        for size in (esz, esz, n * maxv, n * maxv + 1):
            parts.append(raw[o:o + size].copy())
            o += size
        arrays.append((n, maxv, parts, vc))
    want = [gs.mine_collect(db, s, max_edges=me)[0] for db, (_, s, me) in zip(dbs, cases)]
    errors = []

    def worker(t):
        try:
            for rep in range(3):
                i = (t + rep) % len(cases)
                _, s, me = cases[i]
                ext = "lists" if (t + rep) % 2 else "rmpath"
                if t % 2:
                    n, maxv, (e, el, vl, vo), vc = arrays[i]
                    d = gs.Database.from_arrays(n, maxv, e, el, vl, vo, vc, device=True)
                    got, _ = gs.mine_collect(d, s, max_edges=me, extension=ext)
                    d.free()
                else:
                    got, _ = gs.mine_collect(dbs[i], s, max_edges=me, extension=ext)
                if got != want[i]:
                    errors.append((t, rep, i, ext))
        except Exception as exc:  # reported below
            errors.append((t, repr(exc)))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(6)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert errors == []


def test_random_support_counts(gs):
    # gs_support_count (the reference's compute_support_remapped_db_multiple_dfs)
    # on random records against distinct graph ids per key counted with sets:
    # empty input, one key or one graph, unsorted ids and duplicate records
    r = random.Random(77)
    shapes = [(0, 5, 3), (1, 1, 1), (50, 1, 7), (50, 9, 1), (5000, 40, 300), (20000, 700, 5000),
              (100000, 3, 100000)]
    for n, n_keys, n_graphs in shapes:
        keys = [r.randrange(n_keys) for _ in range(n)]
        gids = [r.randrange(n_graphs) for _ in range(n)]
        if n > 10:
            keys += keys[:n // 10]   # duplicate records
            gids += gids[:n // 10]
        sets = [set() for _ in range(n_keys)]
        for k, g in zip(keys, gids):
            sets[k].add(g)
        want = [len(x) for x in sets]
        assert gs.support_count(keys, gids, n_keys, n_graphs) == want, (n, n_keys, n_graphs)
