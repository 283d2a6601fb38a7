"""Full benchmark sizes, checked through size-independent properties (the
oracle cannot mine these sizes in test time):
  * configuration 5 (1,000,000 graphs, 80 M adjacency entries) at minsup 0.5%:
    repeat runs equal, the GPU and host canonicality checks equal, every
    support >= minsup, every pattern's one-edge-shorter prefix present with
    a support at least as large;
  * configuration 3 (64 databases, 916,553 graphs) at minsup 5%: mined as one
    batch equals each database mined alone, and the oracle agrees on the
    smallest databases."""
import os

import pytest

from conftest import run_oracle, to_lines

pytestmark = pytest.mark.gpu


def _properties(gs, pats, minsup):
    sup = {}
    for code, s in pats:
        assert s >= minsup
        sup[code] = s
    for code, s in pats:
        if len(code) > 1:
            parent = code[:-1]
            assert parent in sup and sup[parent] >= s, code


def test_config5_full_size(gs):
    db = gs.Database.generate(5)
    assert len(db) == 1000000
    minsup = 5000
    a, sa = gs.mine_collect(db, minsup)
    b, _ = gs.mine_collect(db, minsup)
    assert a == b and len(a) > 10000
    c, sc = gs.mine_collect(db, minsup, min_check=1)
    assert c == a and sc["min_host_checks"] == sc["candidates"]
    _properties(gs, a, minsup)
    assert sa["min_host_checks"] * 100 <= sa["candidates"]


def test_config3_full_batch(gs, oracle, tmp_path):
    dbs = [gs.Database.generate(3, seed=1000 + i) for i in range(64)]
    sups = [max(1, int(round(0.05 * len(d)))) for d in dbs]
    batch, st = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ)
    assert st["patterns"] == sum(len(b) for b in batch)
    for d, s, got in zip(dbs, sups, batch):
        solo, _ = gs.mine_collect(d, s, label_style=gs.LABELS_SEQ)
        assert got == solo
        _properties(gs, got, s)
    # the oracle on the three smallest databases
    order = sorted(range(64), key=lambda i: len(dbs[i]))[:3]
    for i in order:
        p = str(tmp_path / ("db%d.txt" % i))
        dbs[i].write(p, "txt")
        assert to_lines(batch[i], gs) == run_oracle(oracle, "txt", p, sups[i]), i
