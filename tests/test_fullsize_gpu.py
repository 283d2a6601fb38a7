"""Full benchmark sizes against the oracle's pins (tests/golden/fullsize*.tsv,
made by tests/golden/make_fullsize.py with the oracle mining root-subtree
shares in parallel), plus properties that need no oracle:
  * configuration 5 (1,000,000 graphs, 80 M adjacency entries) at minsup
    0.5%: its pin is checked in test_parity_gpu.py::test_full_size_checksums;
    here repeat runs are equal, the GPU and host canonicality checks agree,
    every support >= minsup and every pattern's one-edge-shorter prefix is
    present with a support at least as large;
  * configuration 3 (64 databases, 916,553 graphs) at minsup 5%: mined as one
    batch, every database's output equals the oracle's pinned count and
    hash, and equals the same database mined alone."""
import hashlib
import os

import pytest

from conftest import GOLDEN, read_lines, to_lines

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
    assert a == b and len(a) == 36572
    c, sc = gs.mine_collect(db, minsup, min_check=1)
    assert c == a and sc["min_host_checks"] == sc["candidates"]
    _properties(gs, a, minsup)
    assert sa["min_host_checks"] * 100 <= sa["candidates"]


def _batch_pins():
    pins = {}
    for line in read_lines(os.path.join(GOLDEN, "fullsize_batch.tsv")):
        if line.startswith("#"):
            continue
        c, seed, scale, dbsha, s, n, sha, me = line.split("\t")
        pins[int(seed)] = (int(s), int(n), sha)
    return pins


def test_config3_full_batch_against_oracle_pins(gs):
    pins = _batch_pins()
    assert sorted(pins) == list(range(1000, 1064))
    dbs = [gs.Database.generate(3, seed=1000 + i) for i in range(64)]
    sups = [max(1, int(round(0.05 * len(d)))) for d in dbs]
    batch, st = gs.mine_batch(dbs, sups, label_style=gs.LABELS_SEQ)
    assert st["patterns"] == sum(len(b) for b in batch)
    for i, (d, s, got) in enumerate(zip(dbs, sups, batch)):
        ps, pn, psha = pins[1000 + i]
        assert s == ps
        lines = to_lines(got, gs)
        assert len(lines) == pn, i
        assert hashlib.sha256(("\n".join(lines) + "\n").encode()).hexdigest() == psha, i
        solo, _ = gs.mine_collect(d, s, label_style=gs.LABELS_SEQ)
        assert got == solo
