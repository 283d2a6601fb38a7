"""gs_support_count_noalloc: the support count for callers that cannot call
cudaMalloc (code inside another framework's memory arena, processes with a
fixed device-memory budget, paths that must avoid the implicit device
synchronisation of cudaMalloc/cudaFree).  It keeps its scratch in a fixed
device array inside the library; the caller hands it device buffers it owns.

Checked through the C ABI against gs_support_count (which allocates) on two
calls in a row, and against distinct graph ids per key counted with Python
sets (records out of range left out); results are integers, so they must be
equal.  This file is collected last on purpose; it passes alone in a fresh
process and after the other tests."""
import ctypes
import random

import pytest

pytestmark = pytest.mark.gpu


def _records(seed, n, n_keys, n_graphs):
    r = random.Random(seed)
    keys = [r.randrange(n_keys) for _ in range(n)]
    gids = sorted(r.randrange(n_graphs) for _ in range(n))
    return keys, gids


def _distinct(keys, gids, n_keys, n_graphs):
    """support[k] = distinct graph ids among the in-range records of key k"""
    sets = [set() for _ in range(n_keys)]
    for k, g in zip(keys, gids):
        if 0 <= k < n_keys and 0 <= g < n_graphs:
            sets[k].add(g)
    return [len(x) for x in sets]


def _call_noalloc(gs, torch, keys, gids, n_keys, n_graphs, out, stream=None):
    dk = torch.tensor(keys if keys else [0], dtype=torch.int32, device="cuda")
    dg = torch.tensor(gids if gids else [0], dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    st = gs.lib().gs_support_count_noalloc(ctypes.c_void_p(dk.data_ptr()), ctypes.c_void_p(dg.data_ptr()),
                                           len(keys), n_keys, n_graphs, ctypes.c_void_p(out.data_ptr()),
                                           ctypes.c_void_p(s))
    assert st == 0, gs.lib().gs_last_error()
    if stream is not None:
        stream.synchronize()  # the call is ordered on that stream alone
    else:
        torch.cuda.synchronize()
    return out.cpu().tolist()


def test_noalloc_matches_allocating_entry_point_twice(gs):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    cases = [(11, 50000, 300, 20000), (12, 30000, 97, 5000)]  # the second call reuses a dirtier scratch
    for seed, n, n_keys, n_graphs in cases:
        keys, gids = _records(seed, n, n_keys, n_graphs)
        want = gs.support_count(keys, gids, n_keys, n_graphs)
        out = torch.full((n_keys,), -1, dtype=torch.int32, device="cuda")
        got = _call_noalloc(gs, torch, keys, gids, n_keys, n_graphs, out)
        assert got == want
        assert got == _distinct(keys, gids, n_keys, n_graphs)


def test_noalloc_against_host_sets(gs):
    torch = pytest.importorskip("torch")
    r = random.Random(5)
    # out-of-range keys and graph ids are ignored
    n_keys, n_graphs = 40, 3000
    keys = [r.randrange(-3, n_keys + 3) for _ in range(20000)]
    gids = [r.randrange(-5, n_graphs + 5) for _ in range(20000)]
    out = torch.full((n_keys,), -1, dtype=torch.int32, device="cuda")
    assert _call_noalloc(gs, torch, keys, gids, n_keys, n_graphs, out) == _distinct(keys, gids, n_keys, n_graphs)
    # no records: every support is 0, after a call that left the scratch dirty
    out = torch.full((n_keys,), -1, dtype=torch.int32, device="cuda")
    assert _call_noalloc(gs, torch, [], [], n_keys, n_graphs, out) == [0] * n_keys
    # no graphs: every record is out of range
    out = torch.full((3,), -1, dtype=torch.int32, device="cuda")
    assert _call_noalloc(gs, torch, [0, 1, 2], [0, 0, 0], 3, 0, out) == [0, 0, 0]
    # an explicit non-default stream, synchronised on its own
    side = torch.cuda.Stream()
    keys, gids = _records(21, 60000, 500, 40000)
    out = torch.full((500,), -1, dtype=torch.int32, device="cuda")
    assert _call_noalloc(gs, torch, keys, gids, 500, 40000, out, stream=side) == _distinct(keys, gids, 500, 40000)
    # the largest bitmap the scratch holds: 32 keys x 32,768 words
    keys, gids = _records(22, 100000, 32, 32768 * 32)
    out = torch.full((32,), -1, dtype=torch.int32, device="cuda")
    assert _call_noalloc(gs, torch, keys, gids, 32, 32768 * 32, out) == _distinct(keys, gids, 32, 32768 * 32)


def test_noalloc_rejects_oversized_bitmaps(gs):
    torch = pytest.importorskip("torch")
    out = torch.zeros(1 << 12, dtype=torch.int32, device="cuda")
    # 4096 keys x 8192 words (262,144 graphs) > 1,048,576 words
    st = gs.lib().gs_support_count_noalloc(None, None, 0, 1 << 12, 1 << 18, ctypes.c_void_p(out.data_ptr()), None)
    assert st == 8  # GS_ERR_LIMIT
    assert b"exceeds" in gs.lib().gs_last_error()
    # host memory for the output is refused
    host = torch.zeros(4, dtype=torch.int32)
    st = gs.lib().gs_support_count_noalloc(None, None, 0, 4, 10, ctypes.c_void_p(host.data_ptr()), None)
    assert st == 1  # GS_ERR_USAGE
    assert b"not device memory" in gs.lib().gs_last_error()
