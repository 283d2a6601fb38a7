"""Device-side ingest of the reference's cudabin arrays
(gs_db_from_arrays_device) against the host conversion (gs_db_from_arrays):
same checks, same database, same mining results."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _cudabin(db, tmp_path):
    p = str(tmp_path / "db.cudabin")
    db.write(p, "cudabin")
    raw = np.fromfile(p, dtype=np.int32)
    n, esz, maxv, vc = (int(x) for x in raw[:4])
    o = 4
    edges = raw[o:o + esz]; o += esz
    elab = raw[o:o + esz]; o += esz
    vlab = raw[o:o + n * maxv]; o += n * maxv
    voff = raw[o:o + n * maxv + 1]
    return n, maxv, edges, elab, vlab, voff, vc


@pytest.mark.parametrize("src", ["cfg1", "gen2", "gen5", "gen3"])
def test_device_ingest_equals_host(gs, tmp_path, src):
    if src == "cfg1":
        db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    else:
        db = gs.Database.generate(int(src[-1]), scale=0.01)
    n, maxv, edges, elab, vlab, voff, vc = _cudabin(db, tmp_path)
    h = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc)
    d = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc, device=True)
    hi, di = h.info(), d.info()
    for k in ("graphs", "vertices", "adjacency_entries", "vertex_labels", "edge_labels"):
        assert hi[k] == di[k], k
    s = max(2, int(0.05 * len(db)))
    a, _ = gs.mine_collect(h, s)
    b, _ = gs.mine_collect(d, s)
    assert a == b and len(a) > 0
    # the host arrays of a device-built database (written back) are the same
    ph, pd = str(tmp_path / "h.txt"), str(tmp_path / "d.txt")
    h.write(ph, "txt")
    d.write(pd, "txt")
    assert open(ph).read() == open(pd).read()


def test_device_ingest_label_values_kept(gs, tmp_path):
    # sparse, negative and large label values map back to themselves
    lines = ["t # 0", "v 0 -7", "v 1 1000", "v 2 -7", "e 0 1 42", "e 1 2 -3",
             "t # 1", "v 0 1000", "v 1 -7", "e 0 1 42"]
    p = tmp_path / "x.txt"
    p.write_text("\n".join(lines) + "\n")
    db = gs.Database.load(str(p), "txt")
    n, maxv, edges, elab, vlab, voff, vc = _cudabin(db, tmp_path)
    d = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc, device=True)
    a, _ = gs.mine_collect(db, 1)
    b, _ = gs.mine_collect(d, 1)
    assert a == b


def test_device_ingest_rejects_what_host_rejects(gs, tmp_path):
    db = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    n, maxv, edges, elab, vlab, voff, vc = _cudabin(db, tmp_path)
    # a self loop: the first entry of graph 0 points back at its own vertex
    e2 = edges.copy()
    e2[voff[0]] = 0
    # an edge that leaves its graph
    e3 = edges.copy()
    e3[voff[0]] = maxv + 1
    # offsets that do not tile the edge array
    v4 = voff.copy()
    v4[1] = v4[2] + 1
    for arrs in ((e2, elab, vlab, voff), (e3, elab, vlab, voff), (edges, elab, vlab, v4)):
        for device in (False, True):
            with pytest.raises(gs.GSpanError) as e:
                gs.Database.from_arrays(n, maxv, *arrs, vc, device=device)
            assert e.value.status == 3, (device, str(e.value))


def test_device_ingest_repeated_pooled(gs, tmp_path):
    # the ingest's scratch and database blocks come from a pool that is kept
    # between ingests: databases of different sizes built, failed, kept alive
    # together and freed out of order all mine as their host conversions do
    srcs = [gs.Database.generate(2, seed=11, scale=0.01),
            gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt"),
            gs.Database.generate(5, seed=12, scale=0.004)]
    arrs = [_cudabin(db, tmp_path) for db in srcs]
    want = []
    for n, maxv, edges, elab, vlab, voff, vc in arrs:
        h = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc)
        want.append(gs.mine_collect(h, max(2, int(0.05 * n)))[0])
        h.free()
    live = {}
    order = [0, 1, 2, 2, 0, 1, 0, 2, 1, 1]
    for step, i in enumerate(order):
        n, maxv, edges, elab, vlab, voff, vc = arrs[i]
        if step % 3 == 1:
            # a failed ingest (self loop) between good ones
            bad = edges.copy()
            bad[voff[0]] = 0
            with pytest.raises(gs.GSpanError):
                gs.Database.from_arrays(n, maxv, bad, elab, vlab, voff, vc, device=True)
        d = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc, device=True)
        assert gs.mine_collect(d, max(2, int(0.05 * n)))[0] == want[i], (step, i)
        if i in live:
            live.pop(i).free()
        live[i] = d
        if step == 5:
            gs.engine_reset()   # also returns the ingest's pooled memory
    for i, d in live.items():
        assert gs.mine_collect(d, max(2, int(0.05 * arrs[i][0])))[0] == want[i]
        d.free()


@pytest.mark.parametrize("hub", [200, 300])
def test_device_ingest_hub_degrees(gs, oracle, tmp_path, hub):
    # a hub vertex with 200-205 entries (the device ingest sorts every
    # vertex's entries, by insertion beyond 8) or 300-305 (beyond its
    # per-thread sort bound of 256: the entries stay in input order and the
    # extension kernels scan every entry): the same patterns as the oracle and
    # the host-built database, the same arrays written back
    import random
    from conftest import run_oracle, to_lines
    r = random.Random(hub)
    lines = []
    for gi in range(6):
        n = hub + 1 + gi
        lines.append("t # %d" % gi)
        lines += ["v %d %d" % (v, r.randrange(3) if v else 0) for v in range(n)]
        edges = [(0, v, r.randrange(2)) for v in range(1, n)]
        edges += [(v, v + 1, 0) for v in range(1, n - 1, 7)]
        lines += ["e %d %d %d" % e for e in edges]
    path = tmp_path / "hub.txt"
    path.write_text("\n".join(lines) + "\n")
    db = gs.Database.load(str(path), "txt")
    n, maxv, edges, elab, vlab, voff, vc = _cudabin(db, tmp_path)
    d = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc, device=True)
    want = run_oracle(oracle, "txt", str(path), 4, ["--max-edges", "2"])
    assert len(want) > 5
    for x in (db, d):
        pats, _ = gs.mine(x, 4, max_edges=2, label_style=gs.LABELS_SEQ)
        assert to_lines(pats, gs) == want
    ph, pd = str(tmp_path / "h.txt"), str(tmp_path / "d.txt")
    db.write(ph, "txt")
    d.write(pd, "txt")
    assert open(ph).read() == open(pd).read()
