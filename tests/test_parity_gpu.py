"""GPU parity: the miner through the C ABI against the reference's golden
outputs and against the oracle on the same seeded inputs.  Bit-exact: same
patterns, same DFS codes, same supports, same order."""
import hashlib
import os

import pytest

from conftest import GOLDEN, golden_runs, read_lines, run_oracle, to_lines

pytestmark = pytest.mark.gpu


def _mine_lines(gs, db, minsup, **kw):
    pats, stats = gs.mine(db, minsup, label_style=gs.LABELS_SEQ, **kw)
    return to_lines(pats, gs), stats


@pytest.mark.parametrize("run", golden_runs(), ids=lambda r: "%s-s%d" % (r[1], r[2]))
def test_golden_parity(gs, run):
    ft, dbf, s, out = run
    db = gs.Database.load(os.path.join(GOLDEN, dbf), ft)
    got, stats = _mine_lines(gs, db, s)
    assert got == read_lines(os.path.join(GOLDEN, out))
    assert stats["launches"] > 0


@pytest.mark.parametrize("wave_nodes", [1, 3, 64])
@pytest.mark.parametrize("minsup", [34, 5])
def test_wave_sizes_agree(gs, wave_nodes, minsup):
    db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    got, stats = _mine_lines(gs, db, minsup, wave_nodes=wave_nodes)
    assert got == read_lines(os.path.join(GOLDEN, "out_cfg1_seed1_s%d.txt" % minsup))
    if wave_nodes == 1:
        assert stats["waves"] == stats["nodes"]


def test_small_waves_by_rows(gs):
    # a tiny row budget splits waves by rows instead of node count
    db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    got, _ = _mine_lines(gs, db, 10, wave_rows=64, wave_words=64)
    assert got == read_lines(os.path.join(GOLDEN, "out_cfg1_seed1_s10.txt"))


def test_full_label_codes(gs):
    db = gs.Database.load(os.path.join(GOLDEN, "fixture_get_labeled_test_database2.txt"), "txt")
    pats, _ = gs.mine(db, 2, label_style=gs.LABELS_FULL)
    seq = []
    for code, sup in pats:
        lab = {}
        for i, (f, t, fl, el, tl) in enumerate(code):
            assert fl != -1 and tl != -1
            if i == 0:
                lab[f] = fl
            assert lab[f] == fl
            if f < t:
                lab[t] = tl
            assert lab[t] == tl
        s = [code[0]] + [(f, t, -1, el, tl if f < t else -1) for f, t, fl, el, tl in code[1:]]
        seq.append("%s\t%d" % (gs.code_to_string(s), sup))
    assert seq == read_lines(os.path.join(GOLDEN, "out_fixture_get_labeled_test_database2_s2.txt"))


@pytest.mark.parametrize("config,scale,minsups", [(2, 0.02, (40, 20)), (5, 0.002, (10,)), (3, 0.05, (None,)),
                                                   (4, 0.02, (None,))])
def test_generated_vs_oracle(gs, oracle, tmp_path, config, scale, minsups):
    db = gs.Database.generate(config, scale=scale)
    p = str(tmp_path / "db.txt")
    db.write(p, "txt")
    for s in minsups:
        s = s or max(2, int(0.05 * len(db)))
        want = run_oracle(oracle, "txt", p, s)
        got, _ = _mine_lines(gs, db, s)
        assert got == want, (config, s)


@pytest.mark.parametrize("nv_range", [(60, 64), (60, 130)])
def test_large_graphs_vs_oracle(gs, oracle, tmp_path, nv_range):
    # graphs around and beyond 64 vertices take the kernels' general
    # membership path (a loop over the row's vertices) instead of a bit set
    import random
    r = random.Random(nv_range[1])
    lines = []
    for gi in range(40):
        nv = r.randint(*nv_range)
        lines.append("t # %d" % gi)
        lines += ["v %d %d" % (v, r.choice([0, 0, 1, 2])) for v in range(nv)]
        edges = set()
        for v in range(1, nv):
            edges.add((r.randrange(v), v))
        for _ in range(nv // 8):
            a, b = r.sample(range(nv), 2)
            edges.add((min(a, b), max(a, b)))
        lines += ["e %d %d %d" % (a, b, r.choice([0, 1])) for a, b in sorted(edges)]
    p = str(tmp_path / "big.txt")
    with open(p, "w") as f:
        f.write("\n".join(lines) + "\n")
    db = gs.Database.load(p, "txt")
    for s in (30, 20):
        want = run_oracle(oracle, "txt", p, s, ["--max-edges", "5"])
        got, _ = _mine_lines(gs, db, s, max_edges=5)
        assert got == want, s


def test_cudabin_and_bin_inputs(gs, tmp_path):
    src = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    want = read_lines(os.path.join(GOLDEN, "out_cfg1_seed1_s17.txt"))
    for ft in ("cudabin", "bin"):
        p = str(tmp_path / ("db." + ft))
        src.write(p, ft)
        got, _ = _mine_lines(gs, gs.Database.load(p, ft), 17)
        assert got == want, ft


@pytest.mark.parametrize("max_edges", [1, 2, 4])
def test_max_edges(gs, oracle, max_edges):
    p = os.path.join(GOLDEN, "cfg1_seed1.txt")
    want = run_oracle(oracle, "txt", p, 10, ["--max-edges", str(max_edges)])
    got, _ = _mine_lines(gs, gs.Database.load(p, "txt"), 10, max_edges=max_edges)
    assert got == want


def test_batch_equals_solo(gs):
    dbs = [gs.Database.generate(3, seed=1000 + i, scale=0.05) for i in range(4)]
    sups = [max(2, int(0.05 * len(d))) for d in dbs]
    batch, stats = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ)
    for d, s, got in zip(dbs, sups, batch):
        solo, _ = gs.mine(d, s, label_style=gs.LABELS_SEQ)
        assert got == solo
    assert stats["patterns"] == sum(len(b) for b in batch)


def test_bulk_output_equals_callbacks(gs):
    db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    cb, _ = gs.mine(db, 10, label_style=gs.LABELS_SEQ)
    bulk, stats = gs.mine_collect(db, 10, label_style=gs.LABELS_SEQ)
    assert bulk == cb
    n, _ = gs.mine_collect(db, 10, decode=False)
    assert n == len(cb) == stats["patterns"]


def test_repeat_is_deterministic(gs):
    db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    a, _ = gs.mine(db, 10)
    b, _ = gs.mine(db, 10)
    assert a == b


def test_minsup_bounds(gs):
    db = gs.Database.load(os.path.join(GOLDEN, "fixture_get_test_database.txt"), "txt")
    with pytest.raises(gs.GSpanError) as e:
        gs.mine(db, len(db))
    assert e.value.status == 6
    with pytest.raises(gs.GSpanError) as e:
        gs.mine(db, 0)
    assert e.value.status == 7
    # the engine stays usable after a rejected call
    got, _ = _mine_lines(gs, db, 9)
    assert got == read_lines(os.path.join(GOLDEN, "out_fixture_get_test_database_s9.txt"))


def _kat(path):
    recs, dfs = [], []
    for line in read_lines(path):
        if line.startswith("#"):
            mvc = int(line.rsplit("=", 1)[1])
            continue
        kind, rest = line.split("\t", 1)
        if kind == "rec":
            recs.append(tuple(int(x) for x in rest.split()))
        else:
            d, s = rest.split("\t")
            dfs.append((tuple(int(x) for x in d.split()), int(s)))
    return recs, dfs, mvc


@pytest.mark.parametrize("name", ["support_kat.tsv", "extract_kat.tsv", "support_mult_block_kat.tsv"])
def test_support_kats(gs, name):
    # records (from, to, fl, el, tl, from_grph, to_grph, row); graph = vertex // max_graph_vertex_count
    recs, dfs, mvc = _kat(os.path.join(GOLDEN, name))
    keys = sorted({r[:5] for r in recs})
    kid = {k: i for i, k in enumerate(keys)}
    sup = gs.support_count([kid[r[:5]] for r in recs], [r[5] // mvc for r in recs], len(keys), 10)
    got = {k: sup[kid[k]] for k in keys}
    assert got == {d: s for d, s in dfs}


def test_support_count_rejects_out_of_range(gs):
    with pytest.raises(gs.GSpanError):
        gs.support_count([0, 5], [0, 0], 2, 4)


def _filter_kat():
    col, recs, res, dfs = [], [], [], None
    for line in read_lines(os.path.join(GOLDEN, "filter_backward_kat.tsv")):
        if line.startswith("#"):
            continue
        tag, rest = line.split("\t")
        vals = tuple(int(x) for x in rest.split())
        if tag == "col":
            col.append(vals)
        elif tag == "rec":
            recs.append(vals)
        elif tag == "dfs":
            dfs = vals
        else:
            res.append(vals)
    return col, recs, dfs, res


def test_filter_backward_kat(gs):
    # filter_backward_embeddings_test.cpp: the last column's rows named by
    # the records of the backward edge (2, 0, 5, 0, 2), in row order
    col, recs, dfs, res = _filter_kat()
    assert gs.filter_backward(col, recs, dfs) == res == [(1, 0), (12, 3), (28, 5)]


def test_filter_backward_random(gs):
    # seeded random columns and records (matching and other edges, rows named
    # twice, records out of row order) against the rows kept in a Python set;
    # an empty column, and an edge no record carries
    import random
    r = random.Random(5)
    edge = (4, 1, 2, 0, 3)
    for n, m in [(0, 0), (1, 3), (50, 40), (5000, 9000), (300000, 200000)]:
        col = [(r.randrange(1 << 30), r.randrange(1 << 20)) for _ in range(n)]
        recs = []
        for _ in range(m if n else 0):
            e = edge if r.random() < 0.4 else (4, r.choice([0, 2, 3]), 2, r.randrange(2), 3)
            recs.append(e + (r.randrange(100), r.randrange(100), r.randrange(n)))
        rows = sorted({x[7] for x in recs if x[:5] == edge})
        assert gs.filter_backward(col, recs, edge) == [col[i] for i in rows], (n, m)
        assert gs.filter_backward(col, recs, (4, 0, 9, 9, 9)) == []


def _fullsize(name="fullsize.tsv"):
    """Rows of a pin table: (config, seed, scale, db sha256, minsup, count, output sha256, max edges)."""
    rows = []
    for line in read_lines(os.path.join(GOLDEN, name)):
        if line.startswith("#"):
            continue
        c, seed, scale, dbsha, s, n, sha, me = line.split("\t")
        rows.append((int(c), int(seed), float(scale), dbsha, int(s), int(n), sha, int(me)))
    return rows


def _sha_lines(lines):
    return hashlib.sha256(("\n".join(lines) + "\n").encode()).hexdigest()


@pytest.mark.parametrize("row", _fullsize(), ids=lambda r: "cfg%d-seed%d-s%d-e%d" % (r[0], r[1], r[4], r[7]))
def test_full_size_checksums(gs, row):
    # the database bytes behind each pin are checked on the CPU
    # (test_host.py::test_pinned_databases_generated_identically)
    config, seed, scale, dbsha, s, n, sha, me = row
    db = gs.Database.generate(config, seed=seed, scale=scale)
    lines, stats = _mine_lines(gs, db, s, max_edges=me)
    assert len(lines) == n
    assert _sha_lines(lines) == sha
    # size-independent properties
    sup = {}
    for line in lines:
        code, v = line.split("\t")
        assert int(v) >= s
        sup[code] = int(v)
    for code, v in sup.items():
        parts = code.split(";")
        if len(parts) > 1:
            parent = ";".join(parts[:-1])
            assert parent in sup and sup[parent] >= v


@pytest.mark.parametrize("config,scale,frac", [(1, 1.0, 0.05), (2, 0.02, 0.02), (3, 0.05, 0.05), (5, 0.002, 0.005)])
def test_gpu_canonicality_matches_host(gs, config, scale, frac):
    # the warp-parallel check decides (nearly) every candidate; the host
    # checker on the same candidates must agree pattern for pattern
    db = gs.Database.generate(config, scale=scale)
    s = max(2, int(frac * len(db)))
    a, sa = gs.mine(db, s, min_check=0)
    b, sb = gs.mine(db, s, min_check=1)
    assert a == b
    assert sb["min_host_checks"] == sb["candidates"]
    assert sa["candidates"] == sb["candidates"]
    assert sa["min_host_checks"] * 10 <= sa["candidates"]


def test_direct_launches_equal_graph_replay(gs):
    db = gs.Database.generate(2, scale=0.02)
    s = max(2, int(0.02 * len(db)))
    a, sa = gs.mine(db, s, launch_mode=0)
    b, sb = gs.mine(db, s, launch_mode=1)
    assert a == b and sa["waves"] == sb["waves"]


def test_deep_wave_contexts_keep_results(gs):
    # a third wave in flight whenever anything is queued (deep_nodes=1) changes
    # how the queue is split into waves, not the patterns
    dbs = [gs.Database.generate(3, seed=1000 + i, scale=0.03) for i in range(4)]
    sups = [max(2, int(0.05 * len(d))) for d in dbs]
    a, sa = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ)
    b, sb = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, deep_nodes=1, wave_nodes=64)
    assert a == b and sa["patterns"] == sb["patterns"]
    lines, _ = _mine_lines(gs, gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt"), 10, deep_nodes=1,
                           wave_nodes=16)
    assert lines == read_lines(os.path.join(GOLDEN, "out_cfg1_seed1_s10.txt"))


def test_one_stream_equals_context_streams(gs):
    # every wave context on the engine's one stream (serial) or each on its
    # own (default): the same waves, patterns and supports
    db = gs.Database.generate(2, scale=0.05)
    s = max(2, int(0.01 * len(db)))
    a, sa = gs.mine(db, s)
    b, sb = gs.mine(db, s, serial=1)
    assert a == b and sa["waves"] == sb["waves"]
    dbs = [gs.Database.generate(3, seed=1000 + i, scale=0.03) for i in range(4)]
    sups = [max(2, int(0.05 * len(d))) for d in dbs]
    c, sc = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, deep_nodes=1, wave_nodes=64)
    d, sd = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, deep_nodes=1, wave_nodes=64, serial=1)
    assert c == d and sc["waves"] == sd["waves"]


def test_batch_split_over_schedulers_keeps_results(gs):
    # the batch split over 1, 2 or 3 schedulers (own engines, own host
    # threads): the same patterns for every database, in batch order
    dbs = [gs.Database.generate(3, seed=1000 + i, scale=0.03) for i in range(7)]
    dbs.append(dbs[2])  # a database twice in one batch
    sups = [max(2, int(0.05 * len(d))) for d in dbs]
    a, sa = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, schedulers=1)
    for p in (2, 3):
        b, sb = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, schedulers=p)
        assert a == b and sa["patterns"] == sb["patterns"]
    assert a[2] == a[7]
    for d, s, pats in zip(dbs, sups, a):
        one, _ = gs.mine(d, s, label_style=gs.LABELS_SEQ)
        assert one == pats


def test_batch_split_reports_a_scheduler_error_and_recovers(gs):
    # a device pool too small for any wave: every scheduler of a split batch
    # fails with GS_ERR_NOMEM, the call reports it, and the engines mine
    # normally again once the limit is lifted
    dbs = [gs.Database.generate(3, seed=1000 + i, scale=0.03) for i in range(16)]
    sups = [max(2, int(0.05 * len(d))) for d in dbs]
    want, _ = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, schedulers=2)
    try:
        gs.engine_reset()
        gs.set_pool_bytes(4096)
        with pytest.raises(gs.GSpanError) as ei:
            gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, schedulers=2)
        assert ei.value.status == 5  # GS_ERR_NOMEM
    finally:
        gs.set_pool_bytes(0)
        gs.engine_reset()
    got, _ = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, schedulers=2)
    assert got == want


def test_one_database_split_by_root_subtrees_keeps_order(gs):
    # one database mined by 2-4 schedulers, each taking every P-th root
    # subtree on its own thread: the same patterns in the reference's order
    db = gs.Database.generate(2, scale=0.1)
    s = max(2, int(0.01 * len(db)))
    a, sa = gs.mine(db, s, label_style=gs.LABELS_SEQ)
    for p in (2, 3, 4):
        b, sb = gs.mine(db, s, label_style=gs.LABELS_SEQ, schedulers=p)
        assert a == b and sa["patterns"] == sb["patterns"]
        c, _ = gs.mine(db, s, label_style=gs.LABELS_SEQ, schedulers=p, root_part=1, root_parts=2)
        d, _ = gs.mine(db, s, label_style=gs.LABELS_SEQ, root_part=1, root_parts=2)
        assert c == d
    lines, _ = _mine_lines(gs, gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt"), 10, schedulers=3)
    assert lines == read_lines(os.path.join(GOLDEN, "out_cfg1_seed1_s10.txt"))


def test_tight_pool_reuses_fenced_blocks(gs):
    # with the device pool capped near the run's peak, blocks released on the
    # host are handed out again only after every stream has passed their last
    # reader (waiting on the fences instead of growing the pool)
    db = gs.Database.generate(2, scale=0.1)
    s = max(2, int(0.01 * len(db)))
    a, sa = gs.mine(db, s)
    try:
        gs.engine_reset()
        gs.set_pool_bytes(max(2 * sa["peak_pool_bytes"], 32 << 20))
        b, sb = gs.mine(db, s)
    finally:
        gs.set_pool_bytes(0)
        gs.engine_reset()
    assert a == b and sb["peak_pool_bytes"] <= max(2 * sa["peak_pool_bytes"], 32 << 20)


def test_autotune_keeps_results(gs):
    dbs = [gs.Database.generate(3, seed=1000 + i, scale=0.05) for i in range(3)]
    sups = [max(2, int(0.05 * len(d))) for d in dbs]
    opts, rep = gs.autotune(dbs, sups)
    assert rep["trials"] >= 10 and rep["best_ms"] <= rep["base_ms"] * 1.05
    assert opts["wave_nodes"] in (1024, 2048, 4096, 8192, 16384)
    a, _ = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ)
    b, _ = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ, **opts)
    assert a == b
