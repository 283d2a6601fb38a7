"""The lists extension strategy (the reference's gspan_cuda_lists): forward
children join their parent's per-row lists of frequent forward extensions
and scan only their new right-most vertex.  It must give exactly the default
strategy's output: the golden outputs, the oracle's, and the default
strategy's on the same inputs (same patterns, codes, supports, order)."""
import os

import pytest

from conftest import GOLDEN, golden_runs, read_lines, run_oracle, to_lines

pytestmark = pytest.mark.gpu


def _lines(gs, db, minsup, **kw):
    pats, stats = gs.mine(db, minsup, label_style=gs.LABELS_SEQ, extension="lists", **kw)
    return to_lines(pats, gs), stats


@pytest.mark.parametrize("run", golden_runs(), ids=lambda r: "%s-s%d" % (r[1], r[2]))
def test_lists_golden_parity(gs, run):
    ft, dbf, s, out = run
    db = gs.Database.load(os.path.join(GOLDEN, dbf), ft)
    got, stats = _lines(gs, db, s)
    want = read_lines(os.path.join(GOLDEN, out))
    assert got == want
    if any(line.count("(") >= 3 for line in want):
        # patterns of three edges come from nodes whose parent kept lists
        assert stats["join_nodes"] > 0 and stats["list_entries"] > 0


@pytest.mark.parametrize("wave_nodes", [1, 3, 64])
def test_lists_wave_sizes(gs, wave_nodes):
    db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    got, _ = _lines(gs, db, 5, wave_nodes=wave_nodes)
    assert got == read_lines(os.path.join(GOLDEN, "out_cfg1_seed1_s5.txt"))


@pytest.mark.parametrize("config,scale,minsups", [(2, 0.02, (40, 20)), (5, 0.002, (10,)), (3, 0.05, (None,)),
                                                   (4, 0.02, (None,))])
def test_lists_generated_vs_oracle(gs, oracle, tmp_path, config, scale, minsups):
    db = gs.Database.generate(config, scale=scale)
    p = str(tmp_path / "db.txt")
    db.write(p, "txt")
    for s in minsups:
        s = s or max(2, int(0.05 * len(db)))
        want = run_oracle(oracle, "txt", p, s)
        got, stats = _lines(gs, db, s)
        assert got == want, (config, s)
        assert stats["join_nodes"] > 0


def test_lists_large_graphs(gs, tmp_path):
    # graphs beyond 64 vertices: the kernels' general membership path
    import random
    r = random.Random(7)
    lines = []
    for gi in range(40):
        nv = r.randint(60, 130)
        lines.append("t # %d" % gi)
        lines += ["v %d %d" % (v, r.choice([0, 0, 1, 2])) for v in range(nv)]
        edges = set()
        for v in range(1, nv):
            edges.add((r.randrange(v), v))
        for _ in range(nv // 8):
            a, b = r.sample(range(nv), 2)
            edges.add((min(a, b), max(a, b)))
        lines += ["e %d %d %d" % (a, b, r.choice([0, 1])) for a, b in sorted(edges)]
    p = tmp_path / "big.txt"
    p.write_text("\n".join(lines) + "\n")
    db = gs.Database.load(str(p), "txt")
    for s in (30, 20):
        want, _ = gs.mine(db, s, label_style=gs.LABELS_SEQ, max_edges=5)
        got, stats = gs.mine(db, s, label_style=gs.LABELS_SEQ, max_edges=5, extension="lists")
        assert got == want, s
        assert stats["join_nodes"] > 0


@pytest.mark.parametrize("max_edges", [2, 3, 4])
def test_lists_max_edges(gs, oracle, max_edges):
    p = os.path.join(GOLDEN, "cfg1_seed1.txt")
    want = run_oracle(oracle, "txt", p, 10, ["--max-edges", str(max_edges)])
    got, _ = _lines(gs, gs.Database.load(p, "txt"), 10, max_edges=max_edges)
    assert got == want


def test_lists_batch_equals_default(gs):
    dbs = [gs.Database.generate(3, seed=1000 + i, scale=0.05) for i in range(4)]
    sups = [max(2, int(0.05 * len(d))) for d in dbs]
    want, _ = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ)
    got, stats = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, extension="lists")
    assert got == want
    assert stats["join_nodes"] > 0


def test_lists_full_configuration_2(gs):
    # 100,000 graphs at minsup 1%, from a fresh engine: its first waves
    # outgrow the initial record buffer, so those waves materialise by
    # re-enumeration and keep no lists (their children scan every vertex),
    # while later waves join
    db = gs.Database.generate(2, scale=1.0)
    gs.engine_reset()
    want, _ = gs.mine_collect(db, 1000)
    gs.engine_reset()
    got, stats = gs.mine_collect(db, 1000, extension="lists")
    assert got == want and len(got) > 1000
    assert stats["join_nodes"] > 0 and stats["list_entries"] > 0


def test_lists_in_the_server(gs):
    # the lists strategy under continuous batching: requests join and leave
    # shared waves (one is cancelled while running) and each result is the
    # default strategy's result for the same request mined alone
    import time
    dbs = [gs.Database.generate(4, seed=2000 + i, scale=0.02 + 0.01 * i) for i in range(3)]
    reqs = [(0, 0.05, 0), (1, 0.02, 5), (2, 0.05, 4), (0, 0.10, 6), (1, 0.05, 0), (2, 0.02, 8)]
    with gs.Server(max_active=8, extension="lists") as srv:
        ids = [srv.add_db(d) for d in dbs]
        rids = []
        for i, (d, f, me) in enumerate(reqs):
            rids.append(srv.submit(ids[d], max(2, int(f * len(dbs[d]))), me))
            if i == 2:
                c = srv.submit(ids[2], max(2, int(0.01 * len(dbs[2]))))
                while srv.status(c) is None and srv.stats()["running"] == 0:
                    time.sleep(0.0005)
                srv.cancel(c)
        got = [srv.result(r) for r in rids]
        _, ic = srv.result(c)
        assert ic["state"] in (gs.REQ_CANCELLED, gs.REQ_DONE)
    for (d, f, me), (pats, info) in zip(reqs, got):
        assert info["state"] == gs.REQ_DONE
        want, _ = gs.mine_collect(dbs[d], max(2, int(f * len(dbs[d]))), max_edges=me)
        assert pats == want


@pytest.mark.parametrize("opts", [dict(launch_mode=1), dict(min_check=1), dict(wave_rows=4096, wave_words=4096),
                                  dict(count_grid=16)], ids=["direct", "host-min", "small-waves", "grid16"])
def test_lists_with_engine_options(gs, opts):
    # the lists strategy under the engine's other options gives the golden output
    db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    got, stats = _lines(gs, db, 5, **opts)
    assert got == read_lines(os.path.join(GOLDEN, "out_cfg1_seed1_s5.txt"))
    assert stats["join_nodes"] > 0


def test_lists_root_partition(gs):
    # root-subtree shares mined with the lists strategy merge into the
    # single-process output
    from gpu_graph_mining_gb300.partition import merge_root_partitions
    db = gs.Database.generate(2, seed=5, scale=0.02)
    s = 40
    want, _ = gs.mine_collect(db, s)
    parts = [gs.mine_collect(db, s, root_part=r, root_parts=3, extension="lists")[0] for r in range(3)]
    assert merge_root_partitions(parts) == want


def test_auto_extension_joins_only_where_the_database_leaves_l2(gs):
    # auto: the lists for waves whose databases' adjacency is larger than
    # three quarters of the L2 (configuration 5 at 0.15 scale: about 145 MB),
    # the plain scan where it stays in L2 (configuration 2 at 0.1 scale)
    big = gs.Database.generate(5, scale=0.15)
    s = max(2, int(round(0.005 * len(big))))
    a, sa = gs.mine(big, s, label_style=gs.LABELS_SEQ)
    b, sb = gs.mine(big, s, label_style=gs.LABELS_SEQ, extension="auto")
    assert a == b and sb["join_nodes"] > 0 and sa["join_nodes"] == 0
    small = gs.Database.generate(2, scale=0.1)
    s = max(2, int(0.01 * len(small)))
    c, _ = gs.mine(small, s, label_style=gs.LABELS_SEQ)
    d, sd = gs.mine(small, s, label_style=gs.LABELS_SEQ, extension="auto")
    assert c == d and sd["join_nodes"] == 0
