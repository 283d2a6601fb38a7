"""Regenerates the golden fixtures in tests/golden/ from the reference.

Run where the reference tree is present (REF=<path>; by default a checkout
named "reference" beside this repository).  It
  * builds the reference's own sequential gSpan (src/gspan) from its sources
    through oracle/Makefile (`make -C oracle ref` -> oracle/_ref/gspan_ref),
  * reads the reference's test sources as text to recover their vectors:
      - src/globals/tests/dfs_ismin_tests.cpp:48-61   canonicality KATs
      - src/globals/test_support.cpp:10-158            three 18-graph fixture databases
      - src/gspan_cuda/tests/compute_support_remapped_test.cpp:23-71  support KAT
      - src/gspan_cuda/tests/extract_extensions_test.cpp:30-157       candidate/support KAT
      - src/gspan_cuda/tests/filter_backward_embeddings_test.cpp:30-131  backward-filter KAT
      - src/gspan_cuda/tests/compute_support_mult_block_test.cpp:15-146 support KAT over two blocks
  * copies the reference's BIN fixture databases (testdata/labeled.bin,
    testdata/unlabeled.bin),
  * writes the synthetic configuration-1 database (seed 1) with this
    package's generator, and
  * runs the reference miner on every fixture database at several supports,
    writing "<code>\\t<support>" lines in the reference's traversal order,
  * builds the reference's convertdb tool (src/globals/convertdb.cpp with its
    fix_database repairs) the same way and runs it on the inputs under
    convert/, keeping its bin and cudabin outputs.

Nothing at test time reads the reference; the tests use only these files.
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
REF = os.environ.get("REF", os.path.abspath(os.path.join(REPO, "..", "reference")))
REF_BIN = os.path.join(REPO, "oracle", "_ref", "gspan_ref")
REF_CONVERT = os.path.join(REPO, "oracle", "_ref", "convertdb_ref")


def build_ref():
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + REF])


def read(path):
    with open(os.path.join(REF, path)) as f:
        return f.read()


def ismin_kats():
    src = read("src/globals/tests/dfs_ismin_tests.cpp")
    body = src[src.index("TEST(dfs_ismin, basic_test)"):]
    body = body[:body.index("/*")]
    out = []
    for line in body.splitlines():
        if line.strip().startswith("//"):
            continue  # commented-out expectations
        m = re.search(r'EXPECT_(TRUE|FALSE)\(static_ismin\("([^"]*)"\)\)', line)
        if m:
            out.append("%s\t%s" % (1 if m.group(1) == "TRUE" else 0, m.group(2)))
    return out


def fixture_dbs():
    src = read("src/globals/test_support.cpp")
    dbs = {}
    for name in ("get_test_database", "get_labeled_test_database", "get_labeled_test_database2"):
        start = src.index("types::graph_database_t %s()" % name)
        arr = src[start:src.index("};", start)]
        codes = [s for s in re.findall(r'"([^"]*)"', arr) if s]
        dbs[name] = codes
    return dbs


def code_to_txt_graph(code_str, gid):
    """DFSCode::toGraph (src/globals/dfs_code.cpp:245-266) written as a txt graph."""
    code = [tuple(int(x) for x in p.strip("()").split()) for p in code_str.split(";")]
    nv = max(max(f, t) for f, t, _, _, _ in code) + 1
    lab = [0] * nv
    for f, t, fl, el, tl in code:
        if fl != -1:
            lab[f] = fl
        if tl != -1:
            lab[t] = tl
    lines = ["t # %d" % gid] + ["v %d %d" % (v, lab[v]) for v in range(nv)]
    lines += ["e %d %d %d" % (f, t, el) for f, t, _, el, _ in code]
    return lines


def support_kat():
    src = read("src/gspan_cuda/tests/compute_support_remapped_test.cpp")
    recs = re.findall(r"extension_element_t\(\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+)\)", src)
    mvc = int(re.search(r"int max_graph_vertex_count = (\d+);", src).group(1))
    dfs = re.findall(r"DFS\((\d+), (\d+), (\d+), (\d+), (\d+)\)", src[src.index("types::DFS dfs_array[]"):])
    exp = re.search(r"int expected_supports \[\] = \{([^}]*)\}", src).group(1)
    return recs, mvc, dfs, [int(x) for x in exp.split(",")]


def mult_block_kat():
    src = read("src/gspan_cuda/tests/compute_support_mult_block_test.cpp")
    recs = re.findall(r"extension_element_t\(\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+)\)", src)
    mvc = int(re.search(r"int max_graph_vertex_count = (\d+);", src).group(1))
    arr = src[src.index("types::DFS dfs_array[]"):]
    arr = arr[:arr.index("};")]
    dfs = re.findall(r"DFS\((\d+), (\d+), (\d+), (\d+), (\d+)\)", arr)
    exp = re.search(r"int expected_supports \[\] = \{([^}]*)\}", src).group(1)
    return recs, mvc, dfs, [int(x) for x in exp.split(",")]


def write_mult_block_kat():
    recs, mvc, dfs, exp = mult_block_kat()
    with open(os.path.join(HERE, "support_mult_block_kat.tsv"), "w") as f:
        f.write("# compute_support_mult_block_test.cpp:15-146: records (from to fl el tl from_grph to_grph row), "
                "max_graph_vertex_count=%d\n" % mvc)
        for r in recs:
            f.write("rec\t%s\n" % " ".join(r))
        for d, e in zip(dfs, exp):
            f.write("dfs\t%s\t%d\n" % (" ".join(d), e))


def extract_kat():
    src = read("src/gspan_cuda/tests/extract_extensions_test.cpp")
    recs = re.findall(r"extension_element_t\(\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+)\)", src)
    mvc = int(re.search(r"int max_graph_vertex_count = (\d+);", src).group(1))
    res = src[src.index("types::DFS dfs_res[]"):]
    dfs = re.findall(r"DFS\((\d+), (\d+), (\d+), (\d+), (\d+)\)", res)
    supp = re.search(r"int supp_res\[\] = \{([^}]*)\}", src).group(1)
    return recs, mvc, dfs, [int(x) for x in supp.split(",")]


def filter_backward_kat():
    src = read("src/gspan_cuda/tests/filter_backward_embeddings_test.cpp")
    body = src[src.index("TEST(filter_backward_embeddings, basic_test)"):]

    def elements(name):
        part = body[body.index(name + "[] = {"):]
        part = part[:part.index("};")]
        return re.findall(r"embedding_element\((-?\d+),\s*(-?\d+)\)", part)

    # the filtered column is the last of the embedding's columns (ptr[])
    cols = re.search(r"embedding_element \*ptr\[\] = \{([^}]*)\}", body).group(1).split(",")
    col = elements(cols[-1].strip())
    recs = re.findall(r"extension_element_t\(\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+),"
                      r"\s*(\d+)\)", body[body.index("exts_array[]"):])
    dfs = re.search(r"types::DFS dfs_elem\((\d+), (\d+), (\d+), (\d+), (\d+)\);", body).groups()
    res = elements("emb_res")
    return col, recs, dfs, res


def write_filter_backward_kat():
    col, recs, dfs, res = filter_backward_kat()
    with open(os.path.join(HERE, "filter_backward_kat.tsv"), "w") as f:
        f.write("# filter_backward_embeddings_test.cpp:30-131: the last embedding column (vertex back_link), the "
                "extension records (from to fl el tl from_grph to_grph row), the backward edge, the filtered column\n")
        for e in col:
            f.write("col\t%s\n" % " ".join(e))
        for r in recs:
            f.write("rec\t%s\n" % " ".join(r))
        f.write("dfs\t%s\n" % " ".join(dfs))
        for e in res:
            f.write("res\t%s\n" % " ".join(e))


def run_ref(ftype, db, minsup, out):
    r = subprocess.run([REF_BIN, ftype, db, str(minsup), out], stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return r.stderr.strip()


def convert_inputs():
    """Inputs for the convertdb runs: graphs needing the fix_database repairs
    (parallel edges, self loops, files numbered from 1), one it cannot repair
    (a parallel edge with another label), and the same repairs in fsg form."""
    d = {}
    d["in_repair.txt"] = ("t # 0\nv 0 1\nv 1 2\nv 2 3\ne 0 1 5\ne 1 0 5\ne 1 2 6\ne 2 2 7\n"
                          "t # 1\nv 0 9\nv 1 1\nv 2 2\ne 1 2 3\n"
                          "t # 2\nv 0 4\nv 1 4\ne 0 1 1\n"
                          "t # 3\nv 0 0\nv 1 5\nv 2 6\nv 3 5\ne 1 2 1\ne 2 3 1\ne 3 1 2\ne 3 2 1\n")
    d["in_conflict.txt"] = "t # 0\nv 0 1\nv 1 2\ne 0 1 5\ne 0 1 6\n"
    d["in_repair.fsg"] = ("t # 0\nv 0 C\nv 1 O\nv 2 N\nu 0 1 s\nu 1 0 s\nu 1 2 d\nu 2 2 s\n"
                          "t # 1\nv 0 H\nv 1 C\nv 2 C\nu 1 2 s\n")
    # the first 40 graphs of the configuration-1 database, made dirty: every
    # 7th graph repeats its first edge and gets a self loop on vertex 1
    lines, g, first = [], -1, None
    with open(os.path.join(HERE, "cfg1_seed1.txt")) as f:
        for line in f:
            line = line.rstrip("\n")
            if line.startswith("t"):
                if g >= 0 and g % 7 == 0 and first:
                    lines += [first, "e 1 1 0"]
                g += 1
                if g == 40:
                    break
                first = None
            elif line.startswith("e") and first is None:
                first = line
            lines.append(line)
    d["in_cfg1_dirty.txt"] = "\n".join(lines) + "\n"
    return d


def convert_runs():
    os.makedirs(os.path.join(HERE, "convert"), exist_ok=True)
    runs = []
    for name, text in convert_inputs().items():
        with open(os.path.join(HERE, "convert", name), "w") as f:
            f.write(text)
        ft = "fsg" if name.endswith(".fsg") else "txt"
        for out_ft in ("bin", "cudabin"):
            out = "out_%s.%s" % (os.path.splitext(name)[0] + ("_fsg" if ft == "fsg" else ""), out_ft)
            path = os.path.join(HERE, "convert", out)
            if os.path.exists(path):
                os.remove(path)
            r = subprocess.run([REF_CONVERT, ft, os.path.join(HERE, "convert", name), out_ft, path],
                               stdout=subprocess.PIPE, stderr=subprocess.PIPE)
            if r.returncode != 0:
                if os.path.exists(path):
                    os.remove(path)
                out = "error"
            runs.append((ft, name, out_ft, out))
    with open(os.path.join(HERE, "convert", "convert_runs.tsv"), "w") as idx:
        idx.write("# input filetype\tinput\toutput filetype\treference convertdb output ('error': it aborted)\n")
        for r in runs:
            idx.write("\t".join(r) + "\n")
            print("convert", *r)


def fsg_molecules(path):
    """A seeded FSG database with string labels (the format whose reader numbers
    labels per graph by first appearance, graph_types.cpp:115-170)."""
    import random
    r = random.Random(5)
    labs = ["C", "O", "N", "S", "Cl"]
    els = ["s", "d", "t"]
    lines = []
    for gi in range(30):
        n = r.randint(4, 14)
        lines.append("t # %d" % gi)
        lines += ["v %d %s" % (v, r.choice(labs)) for v in range(n)]
        seen = set()
        for v in range(1, n):
            a = r.randrange(v)
            seen.add((a, v))
            lines.append("u %d %d %s" % (a, v, r.choice(els)))
        for _ in range(n // 4):
            a, b = sorted(r.sample(range(n), 2))
            if (a, b) not in seen:
                seen.add((a, b))
                lines.append("u %d %d %s" % (a, b, r.choice(els)))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    build_ref()
    fsg_molecules(os.path.join(HERE, "fixture_molecules.fsg"))
    with open(os.path.join(HERE, "ismin_kats.tsv"), "w") as f:
        f.write("# expected(1=min)\tcode   from src/globals/tests/dfs_ismin_tests.cpp:48-61\n")
        f.write("\n".join(ismin_kats()) + "\n")

    for name, codes in fixture_dbs().items():
        lines = []
        for i, c in enumerate(codes):
            lines += code_to_txt_graph(c, i)
        with open(os.path.join(HERE, "fixture_%s.txt" % name), "w") as f:
            f.write("\n".join(lines) + "\n")

    recs, mvc, dfs, exp = support_kat()
    with open(os.path.join(HERE, "support_kat.tsv"), "w") as f:
        f.write("# compute_support_remapped_test.cpp:23-71: records (from to fl el tl from_grph to_grph row), "
                "max_graph_vertex_count=%d\n" % mvc)
        for r in recs:
            f.write("rec\t%s\n" % " ".join(r))
        for d, e in zip(dfs, exp):
            f.write("dfs\t%s\t%d\n" % (" ".join(d), e))
    recs, mvc, dfs, exp = extract_kat()
    with open(os.path.join(HERE, "extract_kat.tsv"), "w") as f:
        f.write("# extract_extensions_test.cpp:30-157: records, then the distinct DFS edges with supports, "
                "max_graph_vertex_count=%d\n" % mvc)
        for r in recs:
            f.write("rec\t%s\n" % " ".join(r))
        for d, e in zip(dfs, exp):
            f.write("dfs\t%s\t%d\n" % (" ".join(d), e))

    write_filter_backward_kat()
    write_mult_block_kat()

    for b in ("labeled.bin", "unlabeled.bin"):
        shutil.copyfile(os.path.join(REF, "testdata", b), os.path.join(HERE, "fixture_" + b))

    sys.path.insert(0, REPO)
    import gpu_graph_mining_gb300 as g
    from gpu_graph_mining_gb300 import build as gb
    gb.build()
    g.Database.generate(1, seed=1).write(os.path.join(HERE, "cfg1_seed1.txt"), "txt")

    runs = []
    for name in ("get_test_database", "get_labeled_test_database", "get_labeled_test_database2"):
        for s in (2, 3, 5, 9):
            runs.append(("txt", "fixture_%s.txt" % name, s))
    for b in ("labeled.bin", "unlabeled.bin"):
        for s in (2, 4, 9):
            runs.append(("bin", "fixture_" + b, s))
    for s in (68, 34, 17, 10, 5):
        runs.append(("txt", "cfg1_seed1.txt", s))
    for s in (3, 5, 8):
        runs.append(("fsg", "fixture_molecules.fsg", s))
    with open(os.path.join(HERE, "golden_runs.tsv"), "w") as idx:
        idx.write("# filetype\tdatabase\tminsup\toutput\treference stderr\n")
        for ft, db, s in runs:
            out = "out_%s_s%d.txt" % (os.path.splitext(db)[0], s)
            log = run_ref(ft, os.path.join(HERE, db), s, os.path.join(HERE, out))
            idx.write("%s\t%s\t%d\t%s\t%s\n" % (ft, db, s, out, log))
            print(ft, db, s, log)
    convert_runs()


if __name__ == "__main__":
    main()
