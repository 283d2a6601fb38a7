"""The reference's own GPU miner, gspan_cuda_no_sort, as a second oracle.

oracle/gspan_cuda.mk builds it for sm_103a from the reference's sources with
the patches CUDA 13 needs (its Fermi-era reduction library replaced by Thrust
versions), into oracle/_ref/gspan_cuda_ref.  Its codes carry full labels and
come in its own traversal order, so each run is compared with the sequential
reference's golden output (or the oracle's) as a sorted set of lines after
the labels are normalised to the sequential convention (fromlabel -1 after
the first edge, tolabel -1 on backward edges).

The reference's GPU code runs only on request: GS_GSPAN_CUDA_REF=1 and the
binary built.  Its hazard H1 applies: the GPU reference sizes label tables
by the number of labels but indexes them by label value, so it needs labels
numbered densely from 0 (on fixture_get_labeled_test_database2, labels up to
200, it aborts).  Its own tests compact the labels first
(src/gspan_cuda/tests/gspan_test.cpp:119); so does this test, order-
preservingly, for a database whose labels are not 0..n-1, mapping the labels
of its output back before the comparison (gSpan only compares labels, so the
patterns are the same up to that map)."""
import os
import subprocess

import pytest

from conftest import GOLDEN, REPO, golden_runs, read_lines, run_oracle

REF_GPU = os.path.join(REPO, "oracle", "_ref", "gspan_cuda_ref")

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("GS_GSPAN_CUDA_REF") != "1" or not os.path.exists(REF_GPU),
                                 reason="the reference's GPU miner runs only on request (GS_GSPAN_CUDA_REF=1, "
                                        "built by oracle/gspan_cuda.mk)")]


def normalise(line):
    """A full-label code line in the sequential miner's label convention."""
    code, sup = line.split("\t")
    out = []
    for i, e in enumerate(code.split(";")):
        f, t, fl, el, tl = (int(x) for x in e.strip("()").split())
        if i > 0:
            fl = -1
        if f > t:
            tl = -1
        out.append("(%d %d %d %d %d)" % (f, t, fl, el, tl))
    return ";".join(out) + "\t" + sup


def _dense_copy(path, tmp_path):
    """(path of a txt copy with labels compacted 0..n-1 in order, vertex map back, edge map back), or
    (path, None, None) when the labels are dense already."""
    lines = read_lines(path)
    vl = sorted({int(x.split()[2]) for x in lines if x.startswith("v ")})
    el = sorted({int(x.split()[3]) for x in lines if x.startswith("e ")})
    if vl == list(range(len(vl))) and el == list(range(len(el))):
        return path, None, None
    vmap, emap = {v: i for i, v in enumerate(vl)}, {e: i for i, e in enumerate(el)}
    out = []
    for x in lines:
        p = x.split()
        if p and p[0] == "v":
            out.append("v %s %d" % (p[1], vmap[int(p[2])]))
        elif p and p[0] == "e":
            out.append("e %s %s %d" % (p[1], p[2], emap[int(p[3])]))
        else:
            out.append(x)
    q = str(tmp_path / "dense.txt")
    with open(q, "w") as f:
        f.write("\n".join(out) + "\n")
    return q, vl, el


def _labels_back(line, vl, el):
    code, sup = line.split("\t")
    out = []
    for e in code.split(";"):
        f, t, fl, l, tl = (int(x) for x in e.strip("()").split())
        out.append("(%d %d %d %d %d)" % (f, t, vl[fl] if fl >= 0 else fl, el[l], vl[tl] if tl >= 0 else tl))
    return ";".join(out) + "\t" + sup


def run_ref_gpu(ftype, path, minsup):
    r = subprocess.run([REF_GPU, ftype, path, str(minsup)], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    # the reference's logger writes its INFO lines to stdout too: patterns are the lines with a tab
    return [normalise(x) for x in r.stdout.splitlines() if "\t" in x]


@pytest.mark.parametrize("run", golden_runs(), ids=lambda r: "%s-s%d" % (r[1], r[2]))
def test_gspan_cuda_matches_golden_set(run, tmp_path):
    ft, db, s, out = run
    if ft == "fsg":
        pytest.skip("per-graph FSG label numbering: labels are not one alphabet")
    path, vl, el = (os.path.join(GOLDEN, db), None, None)
    if ft == "txt":
        path, vl, el = _dense_copy(path, tmp_path)
    got = run_ref_gpu(ft, path, s)
    if vl is not None:
        got = [_labels_back(x, vl, el) for x in got]
    assert sorted(got) == sorted(read_lines(os.path.join(GOLDEN, out)))


@pytest.mark.parametrize("spec,frac", [("2,0,0.05", 0.02), ("5,0,0.01", 0.01), ("3,1003,0.2", 0.05)])
def test_gspan_cuda_matches_oracle_on_generated(oracle, tmp_path, spec, frac):
    p = str(tmp_path / "db.txt")
    subprocess.check_call([oracle, "--write-gen", spec, p])
    n = int(subprocess.check_output([oracle, "--gen-count", spec], text=True))
    s = max(2, int(round(frac * n)))
    assert sorted(run_ref_gpu("txt", p, s)) == sorted(run_oracle(oracle, "txt", p, s))
