"""CPU tests: the oracle against the reference's golden vectors, the C ABI's
exports, canonicality KATs, database I/O and the generators.  No GPU call."""
import hashlib
import json
import os
import re
import subprocess

import pytest

from conftest import GOLDEN, REPO, golden_runs, read_lines, run_oracle

# the reference tree: $REF, by default a checkout named "reference" beside this repository
REF_TREE = os.environ.get("REF", os.path.abspath(os.path.join(REPO, "..", "reference")))


def test_header_symbols_exported(gs):
    with open(os.path.join(REPO, "include", "gspan_gb300.h")) as f:
        hdr = f.read()
    declared = set(re.findall(r"GS_API\s+[^;(]*?\b(gs_\w+)\s*\(", hdr))
    assert declared, "no declarations parsed"
    assert declared == set(gs.EXPORTS)
    lib = gs.lib()
    for name in declared:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", gs.LIB_PATH], stdout=subprocess.PIPE, text=True).stdout
    exported = set(re.findall(r"\b(gs_\w+)$", out, re.M))
    assert declared <= exported


def test_ismin_kats(gs):
    n = 0
    for line in read_lines(os.path.join(GOLDEN, "ismin_kats.tsv")):
        if line.startswith("#"):
            continue
        exp, code = line.split("\t")
        assert gs.dfs_code_is_min(gs.parse_code(code)) == (exp == "1"), code
        n += 1
    assert n == 12


@pytest.mark.parametrize("run", golden_runs(), ids=lambda r: "%s-s%d" % (r[1], r[2]))
def test_oracle_matches_reference_golden(oracle, run):
    ft, db, s, out = run
    got = run_oracle(oracle, ft, os.path.join(GOLDEN, db), s)
    assert got == read_lines(os.path.join(GOLDEN, out))


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF_TREE, "testdata", "Chemical_340")),
                    reason="reference tree not present")
@pytest.mark.parametrize("minsup", [68, 34])
def test_oracle_matches_reference_binary_on_chemical340(oracle, minsup):
    ref = os.path.join(REPO, "oracle", "_ref", "gspan_ref")
    if not os.path.exists(ref):
        subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref"])
    path = os.path.join(REF_TREE, "testdata", "Chemical_340")
    want = run_oracle(ref, "txt", path, minsup)
    got = run_oracle(oracle, "txt", path, minsup)
    assert got == want


def test_oracle_time_limit_gives_prefix(oracle):
    full = run_oracle(oracle, "txt", os.path.join(GOLDEN, "cfg1_seed1.txt"), 5)
    part = run_oracle(oracle, "txt", os.path.join(GOLDEN, "cfg1_seed1.txt"), 5, ["--time-limit", "0.000001"])
    assert full[:len(part)] == part


def test_oracle_exit_codes(oracle):
    db = os.path.join(GOLDEN, "fixture_get_test_database.txt")
    assert subprocess.run([oracle, "txt", db, "18"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode == 2
    assert subprocess.run([oracle, "txt", db, "0"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode == 3


def _canon(db_path, ftype, gs):
    """Order-free form of a database: per graph, vertex labels and sorted edge triples."""
    tmp = db_path + ".canon.txt"
    gs.Database.load(db_path, ftype).write(tmp, "txt")
    graphs, cur = [], None
    for line in read_lines(tmp):
        p = line.split()
        if p[0] == "t":
            cur = ([], [])
            graphs.append(cur)
        elif p[0] == "v":
            cur[0].append(int(p[2]))
        elif p[0] == "e":
            a, b, l = int(p[1]), int(p[2]), int(p[3])
            cur[1].append((min(a, b), max(a, b), l))
    os.remove(tmp)
    return [(tuple(v), tuple(sorted(e))) for v, e in graphs]


@pytest.mark.parametrize("ftype", ["txt", "bin", "cudabin"])
def test_database_roundtrip(gs, tmp_path, ftype):
    src = os.path.join(GOLDEN, "cfg1_seed1.txt")
    d = gs.Database.load(src, "txt")
    out = str(tmp_path / ("db." + ftype))
    d.write(out, ftype)
    assert _canon(src, "txt", gs) == _canon(out, ftype, gs)
    assert len(gs.Database.load(out, ftype)) == len(d) == 340


def test_bin_fixture_matches_txt_fixture(gs):
    # testdata/labeled.bin serialises the labeled test database (test_support.cpp)
    a = _canon(os.path.join(GOLDEN, "fixture_labeled.bin"), "bin", gs)
    b = _canon(os.path.join(GOLDEN, "fixture_get_labeled_test_database.txt"), "txt", gs)
    assert a == b


def test_from_arrays_matches_cudabin_file(gs, tmp_path):
    import numpy as np
    d = gs.Database.load(os.path.join(GOLDEN, "cfg1_seed1.txt"), "txt")
    p = str(tmp_path / "c.cudabin")
    d.write(p, "cudabin")
    raw = np.fromfile(p, dtype=np.int32)
    n, esz, maxv, vc = raw[:4]
    o = 4
    edges = raw[o:o + esz]; o += esz
    elab = raw[o:o + esz]; o += esz
    vlab = raw[o:o + n * maxv]; o += n * maxv
    voff = raw[o:o + n * maxv + 1]
    d2 = gs.Database.from_arrays(n, maxv, edges, elab, vlab, voff, vc)
    assert d2.info()["adjacency_entries"] == d.info()["adjacency_entries"]
    assert d2.info()["vertices"] == d.info()["vertices"]


def test_fsg_labels_renumbered_per_graph(gs, tmp_path):
    # Graph::read_fsg numbers string labels per graph by first appearance
    p = tmp_path / "x.fsg"
    p.write_text("t # 0\nv 0 C\nv 1 O\nu 0 1 s\nt # 1\nv 0 O\nv 1 C\nu 0 1 d\n")
    d = gs.Database.load(str(p), "fsg")
    out = tmp_path / "x.txt"
    d.write(str(out), "txt")
    assert read_lines(str(out)) == ["t # 0", "v 0 0", "v 1 1", "e 0 1 0", "t # 1", "v 0 0", "v 1 1", "e 0 1 0"]


def test_load_errors(gs, tmp_path):
    with pytest.raises(gs.GSpanError) as e:
        gs.Database.load(str(tmp_path / "missing.txt"), "txt")
    assert e.value.status == 2
    p = tmp_path / "loop.txt"
    p.write_text("t # 0\nv 0 1\nv 1 1\ne 0 0 1\n")
    with pytest.raises(gs.GSpanError) as e:
        gs.Database.load(str(p), "txt")
    assert e.value.status == 3
    p = tmp_path / "par.txt"
    p.write_text("t # 0\nv 0 1\nv 1 1\ne 0 1 1\ne 1 0 2\n")
    with pytest.raises(gs.GSpanError) as e:
        gs.Database.load(str(p), "txt")
    assert e.value.status == 3
    p = tmp_path / "order.txt"
    p.write_text("t # 0\nv 0 1\ne 0 1 1\nv 1 1\n")
    with pytest.raises(gs.GSpanError):
        gs.Database.load(str(p), "txt")
    with pytest.raises(ValueError):
        gs.filetype("xml")


def test_generator_deterministic(gs, tmp_path):
    a, b = str(tmp_path / "a.txt"), str(tmp_path / "b.txt")
    gs.Database.generate(2, seed=7, scale=0.01).write(a)
    gs.Database.generate(2, seed=7, scale=0.01).write(b)
    assert open(a).read() == open(b).read()
    c = str(tmp_path / "c.txt")
    gs.Database.generate(2, seed=8, scale=0.01).write(c)
    assert open(a).read() != open(c).read()
    # the committed configuration-1 fixture is what the generator makes
    gs.Database.generate(1, seed=1).write(c)
    assert hashlib.sha256(open(c, "rb").read()).hexdigest() == \
        hashlib.sha256(open(os.path.join(GOLDEN, "cfg1_seed1.txt"), "rb").read()).hexdigest()


@pytest.mark.parametrize("config,seed,scale", [(1, 1, 1.0), (2, 0, 0.01), (2, 9, 0.005), (3, 1000, 0.05),
                                               (3, 1041, 0.02), (4, 2003, 0.01), (5, 0, 0.002), (5, 77, 0.001)])
def test_oracle_generator_matches_product_generator(gs, oracle, tmp_path, config, seed, scale):
    # the oracle makes the benchmark databases itself (the timed CPU arm and
    # the full-size pins load nothing of the package): same bytes as txt
    a, b = str(tmp_path / "o.txt"), str(tmp_path / "p.txt")
    subprocess.check_call([oracle, "--write-gen", "%d,%d,%r" % (config, seed, scale), a])
    gs.Database.generate(config, seed=seed, scale=scale).write(b)
    assert open(a, "rb").read() == open(b, "rb").read()
    n = int(subprocess.check_output([oracle, "--gen-count", "%d,%d,%r" % (config, seed, scale)], text=True))
    assert n == len(gs.Database.generate(config, seed=seed, scale=scale))


def test_oracle_generator_matches_pinned_checksums(oracle, tmp_path):
    # the committed configuration-1 fixture and the full-size databases'
    # checksums in the pin tables (configuration 2: 100,000 graphs)
    p = str(tmp_path / "c1.txt")
    subprocess.check_call([oracle, "--write-gen", "1", p])
    assert open(p, "rb").read() == open(os.path.join(GOLDEN, "cfg1_seed1.txt"), "rb").read()
    rows = [r.split("\t") for r in read_lines(os.path.join(GOLDEN, "fullsize.tsv")) if not r.startswith("#")]
    for c, seed, scale, dbsha in {tuple(r[:4]) for r in rows if r[0] == "2"}:
        subprocess.check_call([oracle, "--write-gen", "%s,%s,%s" % (c, seed, scale), p])
        assert hashlib.sha256(open(p, "rb").read()).hexdigest() == dbsha


def _pin_rows():
    rows = []
    for name in ("fullsize.tsv", "fullsize_batch.tsv"):
        for line in read_lines(os.path.join(GOLDEN, name)):
            if not line.startswith("#"):
                c, seed, scale, dbsha = line.split("\t")[:4]
                rows.append((int(c), int(seed), float(scale), dbsha))
    return sorted(set(rows))


def test_pinned_databases_generated_identically(gs, tmp_path):
    # the GPU tests regenerate the pinned full-size databases with the
    # package's generator: the bytes must be the ones the oracle mined
    rows = _pin_rows()
    assert len(rows) >= 66  # configurations 2 and 5, the 64 batch databases, the serving databases
    p = str(tmp_path / "db.txt")
    for c, seed, scale, dbsha in rows:
        gs.Database.generate(c, seed=seed, scale=scale).write(p)
        h = hashlib.sha256()
        with open(p, "rb") as f:
            for blk in iter(lambda: f.read(1 << 24), b""):
                h.update(blk)
        assert h.hexdigest() == dbsha, (c, seed, scale)
    os.remove(p)


def test_oracle_gen_input_equals_txt_input(oracle, tmp_path):
    p = str(tmp_path / "d.txt")
    subprocess.check_call([oracle, "--write-gen", "2,4,0.01", p])
    assert run_oracle(oracle, "gen", "2,4,0.01", 30) == run_oracle(oracle, "txt", p, 30)


def test_reference_arm_loads_nothing_of_the_package(oracle):
    # bench.py --impl reference times the oracle only: the package (and its
    # native library) must not be imported in that process
    code = ("import runpy, sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--scale', '0.002', "
            "'--steps', '2', '--warmup', '1', '--ref-seconds', '0.2']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "assert not [m for m in sys.modules if m.startswith('gpu_graph_mining_gb300')], 'package imported'")
    r = subprocess.run(["python", "-c", code], cwd=REPO, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 2
    assert line["config"]["graphs"] == 2000 and line["config"]["minsup"] == 10


def test_generator_shapes(gs):
    i = gs.Database.generate(2, scale=0.02).info()
    assert i["graphs"] == 2000 and i["vertex_labels"] == 5 and i["edge_labels"] == 5
    mean_edges = i["adjacency_entries"] / 2 / i["graphs"]
    assert 27 < mean_edges < 34
    i = gs.Database.generate(5, scale=0.001).info()
    assert i["graphs"] == 1000 and i["vertex_labels"] == 10 and i["edge_labels"] == 3
    i = gs.Database.generate(1).info()
    assert i["graphs"] == 340 and i["edge_labels"] == 4


def test_cli_exit_codes(gs):
    db = os.path.join(GOLDEN, "fixture_get_test_database.txt")
    r = subprocess.run([gs.CLI_PATH], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    assert r.returncode == 1
    r = subprocess.run([gs.CLI_PATH, "txt", db, "18"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    assert r.returncode == 2
    r = subprocess.run([gs.CLI_PATH, "txt", db, "0"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    assert r.returncode == 3


def test_server_validates_requests_on_the_host(gs):
    # argument checks need no GPU: nothing is admitted
    db = gs.Database.load(os.path.join(GOLDEN, "fixture_get_test_database.txt"), "txt")
    with gs.Server() as srv:
        d = srv.add_db(db)
        with pytest.raises(gs.GSpanError) as e:
            srv.submit(d + 1, 2)
        assert e.value.status == 1
        with pytest.raises(gs.GSpanError) as e:
            srv.submit(d, 0)
        assert e.value.status == 7
        with pytest.raises(gs.GSpanError) as e:
            srv.submit(d, len(db))
        assert e.value.status == 6
        with pytest.raises(gs.GSpanError) as e:
            srv.result(12345, timeout_ms=0)
        assert e.value.status == 1
        s = srv.stats()
        assert s["submitted"] == 0 and s["running"] == 0


@pytest.mark.parametrize("name", ["support_kat.tsv", "extract_kat.tsv", "support_mult_block_kat.tsv"])
def test_support_kat_fixtures_restated(name):
    # the expected supports of the reference's support KATs equal the distinct
    # graphs (from_grph // max_graph_vertex_count) among each edge's records
    recs, want = [], {}
    for line in read_lines(os.path.join(GOLDEN, name)):
        if line.startswith("#"):
            mvc = int(line.rsplit("=", 1)[1])
            continue
        kind, rest = line.split("\t", 1)
        if kind == "rec":
            recs.append(tuple(int(x) for x in rest.split()))
        else:
            d, sup = rest.split("\t")
            want[tuple(int(x) for x in d.split())] = int(sup)
    got = {d: len({r[5] // mvc for r in recs if r[:5] == d}) for d in want}
    assert got == want and len(want) >= 5


def test_filter_backward_kat_fixture_restated():
    # the reference's filter KAT: the last column's rows named by the records
    # of the backward edge, in row order
    col, recs, res, dfs = [], [], [], None
    for line in read_lines(os.path.join(GOLDEN, "filter_backward_kat.tsv")):
        if line.startswith("#"):
            continue
        tag, rest = line.split("\t")
        vals = tuple(int(x) for x in rest.split())
        {"col": col, "rec": recs, "res": res}.get(tag, []).append(vals)
        if tag == "dfs":
            dfs = vals
    rows = sorted({r[7] for r in recs if r[:5] == dfs})
    assert [col[i] for i in rows] == res and len(res) == 3


def test_filter_backward_validates_on_the_host(gs):
    # argument checks before any device work: a forward edge (the reference
    # aborts), a matching record naming a row outside the column
    col = [(1, 0), (4, 1)]
    with pytest.raises(gs.GSpanError) as e:
        gs.filter_backward(col, [(0, 1, 0, 0, 0, 0, 0, 0)], (0, 1, 0, 0, 0))
    assert e.value.status == 1
    with pytest.raises(gs.GSpanError) as e:
        gs.filter_backward(col, [(2, 0, 5, 0, 2, 0, 0, 2)], (2, 0, 5, 0, 2))
    assert e.value.status == 1
    assert gs.filter_backward([], [], (2, 0, 5, 0, 2)) == []


def _convert_runs():
    rows = []
    for line in read_lines(os.path.join(GOLDEN, "convert", "convert_runs.tsv")):
        if not line.startswith("#"):
            rows.append(tuple(line.split("\t")))
    return rows


@pytest.mark.parametrize("run", _convert_runs(), ids=lambda r: "%s-%s" % (r[1], r[2]))
def test_convert_matches_reference_tool(gs, tmp_path, run):
    # outputs of the reference's convertdb (with fix_database), byte for byte
    ft, name, out_ft, out = run
    dst = str(tmp_path / ("x." + out_ft))
    src = os.path.join(GOLDEN, "convert", name)
    if out == "error":
        with pytest.raises(gs.GSpanError) as e:
            gs.convert_database(src, ft, dst, out_ft)
        assert e.value.status == 3 and "different label" in str(e.value)
        return
    info = gs.convert_database(src, ft, dst, out_ft)
    with open(dst, "rb") as a, open(os.path.join(GOLDEN, "convert", out), "rb") as b:
        assert a.read() == b.read()
    assert info["graphs"] >= 1
    # the repaired database is simple: it loads and mines
    d = gs.Database.load(dst, out_ft)
    assert len(d) == info["graphs"]


def test_convertdb_cli(gs, tmp_path):
    exe = os.path.join(os.path.dirname(gs.LIB_PATH), "gspan_gb300_convertdb")
    r = subprocess.run([exe, "txt"], stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 1
    dst = str(tmp_path / "o.cudabin")
    src = os.path.join(GOLDEN, "convert", "in_repair.txt")
    r = subprocess.run([exe, "txt", src, "cudabin", dst], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0 and "repaired 2" in r.stdout
    with open(dst, "rb") as a, open(os.path.join(GOLDEN, "convert", "out_in_repair.cudabin"), "rb") as b:
        assert a.read() == b.read()
    r = subprocess.run([exe, "txt", os.path.join(GOLDEN, "convert", "in_conflict.txt"), "bin", dst],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 2


@pytest.mark.skipif(not os.path.exists(os.path.join(REPO, "oracle", "_ref", "convertdb_ref")),
                    reason="the reference's convertdb is built only where the reference tree is")
def test_convert_live_against_reference_tool(gs, tmp_path):
    # a larger dirty database: every 3rd graph of configuration 1 gets a repeated
    # edge, every 5th a self loop, and every 4th is shifted to ids from 1
    import random
    rnd = random.Random(5)
    src = gs.Database.generate(1, seed=9, scale=0.5)
    p = str(tmp_path / "clean.txt")
    src.write(p, "txt")
    out, g, edges = [], -1, []
    for line in read_lines(p):
        if line.startswith("t"):
            g += 1
            out.append(line)
            continue
        parts = line.split()
        if g % 4 == 0:
            parts[1] = str(int(parts[1]) + 1)
            if parts[0] == "e":
                parts[2] = str(int(parts[2]) + 1)
            if parts[0] == "v" and parts[1] == "1":
                out.append("v 0 %d" % rnd.randint(0, 3))
        out.append(" ".join(parts))
        if parts[0] == "e" and g % 3 == 0 and rnd.random() < 0.3:
            out.append("e %s %s %s" % (parts[2], parts[1], parts[3]))
        if parts[0] == "e" and g % 5 == 0 and rnd.random() < 0.1:
            out.append("e %s %s 1" % (parts[1], parts[1]))
    dirty = str(tmp_path / "dirty.txt")
    with open(dirty, "w") as f:
        f.write("\n".join(out) + "\n")
    ref = os.path.join(REPO, "oracle", "_ref", "convertdb_ref")
    for ft in ("bin", "cudabin"):
        a, b = str(tmp_path / ("a." + ft)), str(tmp_path / ("b." + ft))
        subprocess.run([ref, "txt", dirty, ft, a], check=True, stdout=subprocess.DEVNULL)
        gs.convert_database(dirty, "txt", b, ft)
        assert open(a, "rb").read() == open(b, "rb").read(), ft


def test_option_structs_match_the_header(gs):
    # the ctypes mirrors of gs_mine_opts / gs_mine_stats against the header's
    # field lists, and the extension option's defaults and spellings
    import ctypes
    import re
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "gspan_gb300.h")).read()
    for cname, py in (("gs_mine_opts", gs.MineOpts), ("gs_mine_stats", gs.MineStats),
                      ("gs_server_opts", gs.ServerOpts)):
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (cname, cname), hdr, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        names = re.findall(r"\b(?:int32_t|int64_t|double)\s+(\w+);", body)
        assert names == [f for f, _ in py._fields_], cname
    o = gs.MineOpts()
    gs.lib().gs_mine_opts_default(ctypes.byref(o))
    assert o.extension == gs.EXTENSION_RMPATH
    assert gs._opts().extension == gs.EXTENSION_RMPATH
    assert gs._opts(extension="auto").extension == gs.EXTENSION_AUTO
    assert gs._opts(extension="lists").extension == gs.EXTENSION_LISTS
    assert gs._opts(extension="rmpath").extension == gs.EXTENSION_RMPATH
    with pytest.raises(ValueError):
        gs._opts(extension="bogus")
    # gs_tune_report too, and every option the autotuner returns is a keyword
    # of mine() (the bench passes the tuned options to single-database calls)
    body = re.search(r"typedef struct gs_tune_report \{(.*?)\} gs_tune_report;", hdr, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    assert re.findall(r"\b(?:int32_t|int64_t|double)\s+(\w+);", body) == [f for f, _ in gs.TuneReport._fields_]
    import inspect
    params = set(inspect.signature(gs.mine).parameters) & set(inspect.signature(gs._opts).parameters)
    for f, _ in gs.MineOpts._fields_:
        assert f in params, f


def test_drop_in_shim_compiles_against_the_reference(tmp_path):
    # the C++ drop-in (a gspan_cuda::gspan_cuda subclass and the
    # get_gspan_cuda_instance factory) compiled with the reference's own
    # headers and flags (nvcc -x cu), as a maintainer links it into the mains
    src = os.path.join(REF_TREE, "src")
    if not os.path.isdir(os.path.join(src, "gspan_cuda")):
        pytest.skip("reference tree not present")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = ["nvcc", "-x", "cu", "-std=c++17", "-DLOG_INFO", "-DSTLPORT_UNAVAL",
           "-gencode", "arch=compute_103a,code=sm_103a"]
    cmd += ["-I" + os.path.join(src, d) for d in ("gspan_cuda", "globals", "cuda_pp", "reduction")]
    cmd += ["-I" + os.path.join(repo, "include"), "-c",
            os.path.join(repo, "gpu_graph_mining_gb300", "shim", "gspan_cuda_shim.cpp"),
            "-o", str(tmp_path / "shim.o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    nm = subprocess.run(["nm", "-C", str(tmp_path / "shim.o")], capture_output=True, text=True).stdout
    assert "get_gspan_cuda_instance()" in nm
    for sym in ("gs_db_from_arrays_device", "gs_mine", "gs_db_free", "gs_last_error"):
        assert sym in nm, sym


def test_bench_roofline_and_traffic_helpers():
    # the bench line's roofline block from kernel-side counters: the count
    # kernel on top, the others beside it, their exclusive (one-stream) times,
    # and the committed DRAM/algorithmic ratio applied per launch
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(REPO, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    st = {"count_bytes": 2.0e11, "count_ms": 100.0, "mat_bytes": 9.0e10, "mat_ms": 20.0, "sel_bytes": 1.5e9,
          "sel_ms": 3.0, "min_ms": 2.5, "waves": 110}
    ser = dict(st, count_ms=90.0)
    r = b.roofline([st, st], 6700.0, "measured", None, None, [ser])
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["kernel"] == "k_wave count"
    assert abs(r["achieved"] - 2000.0) < 1e-6 and abs(r["frac"] - 2000.0 / 6700.0) < 1e-12
    assert r["launches_per_step"] == 110
    assert set(r["kernels"]) == set(r["kernels_one_stream"])
    assert abs(r["kernels_one_stream"]["k_wave count"]["achieved"] - 2.0e11 / 0.09 / 1e9) < 1e-6
    t, note = b.count_traffic("config5", 2.0e11, 100)
    ratio = json.load(open(os.path.join(REPO, "profiles", "k_wave_count_traffic_config5.json")))
    expect = ratio["dram_bytes_per_pass"] / ratio["algorithmic_bytes_per_pass"] * 2.0e9
    assert abs(t - expect) < 1.0 and "k_wave_count_traffic_config5.json" in note
    assert b.count_traffic("nonexistent", 1.0, 1) == (None, None)
