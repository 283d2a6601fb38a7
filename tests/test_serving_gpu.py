"""Serving (gs_server_*): requests that arrive while others are mined join
their waves (continuous batching); each request's result must be the same
as the same request mined alone, bit for bit and in the same order."""
import time

import pytest

pytestmark = pytest.mark.gpu


def _dbs(gs):
    return [gs.Database.generate(4, seed=2000 + i, scale=0.02 + 0.01 * i) for i in range(3)]


def _solo(gs, db, minsup, max_edges):
    pats, _ = gs.mine_collect(db, minsup, max_edges=max_edges)
    return pats


def test_results_same_alone_and_in_the_mix(gs):
    dbs = _dbs(gs)
    reqs = [(0, 0.05, 0), (1, 0.02, 5), (2, 0.05, 4), (0, 0.10, 6), (1, 0.05, 0), (2, 0.02, 8),
            (0, 0.02, 0), (1, 0.10, 4)]
    with gs.Server(max_active=8) as srv:
        ids = [srv.add_db(d) for d in dbs]
        rids = []
        # a first group, then more while those are on the GPU
        for i, (d, f, me) in enumerate(reqs):
            rids.append(srv.submit(ids[d], max(2, int(f * len(dbs[d]))), me))
            if i == 3:
                time.sleep(0.002)
        got = [srv.result(r) for r in rids]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for (d, f, me), (pats, info) in zip(reqs, got):
        assert info["state"] == gs.REQ_DONE
        want = _solo(gs, dbs[d], max(2, int(f * len(dbs[d]))), me)
        assert pats == want
        assert info["patterns"] == len(want)


def test_overlapping_requests_share_waves(gs):
    # submitted together with room for all: they are admitted at once
    dbs = _dbs(gs)
    with gs.Server(max_active=16) as srv:
        ids = [srv.add_db(d) for d in dbs]
        rids = [srv.submit(ids[i % 3], max(2, int(0.02 * len(dbs[i % 3])))) for i in range(6)]
        for r in rids:
            srv.result(r)
        st = srv.stats()
    assert st["max_running"] > 1


def test_budget_limits_admission(gs):
    # a budget below any one request's estimate admits one request at a time
    dbs = _dbs(gs)
    with gs.Server(budget_bytes=1, max_active=16) as srv:
        ids = [srv.add_db(d) for d in dbs]
        rids = [srv.submit(ids[i % 3], max(2, int(0.05 * len(dbs[i % 3])))) for i in range(5)]
        res = [srv.result(r) for r in rids]
        st = srv.stats()
    assert st["max_running"] == 1 and st["completed"] == 5
    for i, (pats, info) in enumerate(res):
        assert pats == _solo(gs, dbs[i % 3], max(2, int(0.05 * len(dbs[i % 3]))), 0)


def test_cancel(gs):
    dbs = _dbs(gs)
    with gs.Server(max_active=1) as srv:
        ids = [srv.add_db(d) for d in dbs]
        a = srv.submit(ids[2], max(2, int(0.01 * len(dbs[2]))))
        b = srv.submit(ids[0], max(2, int(0.05 * len(dbs[0]))))
        srv.cancel(b)              # still queued behind a (one active slot)
        pa, ia = srv.result(a)
        pb, ib = srv.result(b)
        assert ib["state"] == gs.REQ_CANCELLED and pb is None
        assert ia["state"] == gs.REQ_DONE
        assert pa == _solo(gs, dbs[2], max(2, int(0.01 * len(dbs[2]))), 0)
        # a running request stops at its next wave and the server goes on
        c = srv.submit(ids[2], max(2, int(0.01 * len(dbs[2]))))
        while srv.status(c) is None and srv.stats()["running"] == 0:
            time.sleep(0.0005)
        srv.cancel(c)
        pc, ic = srv.result(c)
        assert ic["state"] in (gs.REQ_CANCELLED, gs.REQ_DONE)
        d = srv.submit(ids[1], max(2, int(0.05 * len(dbs[1]))))
        pd, idd = srv.result(d)
        assert pd == _solo(gs, dbs[1], max(2, int(0.05 * len(dbs[1]))), 0)
        st = srv.stats()
    assert st["cancelled"] >= 1
