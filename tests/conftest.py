"""Shared fixtures.  Tests marked `gpu` need a GB300; everything else runs on CPU."""
import os
import subprocess
import sys

import pytest

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
GOLDEN = os.path.join(REPO, "tests", "golden")
ORACLE = os.path.join(REPO, "oracle", "_build", "gspan_oracle")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def gs():
    """The package with its native library built."""
    from gpu_graph_mining_gb300 import build as b
    b.build()
    import gpu_graph_mining_gb300 as g
    g.lib()
    return g


@pytest.fixture(scope="session")
def oracle():
    """Path of the CPU restatement of the reference's sequential gSpan (the checker)."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle")])
    return ORACLE


def run_oracle(oracle_bin, ftype, path, minsup, extra=()):
    """Runs the checker; returns its output lines ('<code>\\t<support>')."""
    r = subprocess.run([oracle_bin, ftype, path, str(minsup)] + list(extra), stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout.splitlines()


def golden_runs():
    """(filetype, database file, minsup, output file) of every golden run."""
    out = []
    with open(os.path.join(GOLDEN, "golden_runs.tsv")) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            ft, db, s, o = line.rstrip("\n").split("\t")[:4]
            out.append((ft, db, int(s), o))
    return out


def read_lines(path):
    with open(path) as f:
        return f.read().splitlines()


def to_lines(patterns, g):
    return ["%s\t%d" % (g.code_to_string(c), s) for c, s in patterns]
