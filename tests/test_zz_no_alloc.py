"""gs_support_count_noalloc: the support count for callers that cannot call
cudaMalloc (code inside another framework's memory arena, processes with a
fixed device-memory budget, paths that must avoid the implicit device
synchronisation of cudaMalloc/cudaFree).  It keeps its scratch in a fixed
device array inside the library; the caller hands it device buffers it owns.

Checked through the C ABI against gs_support_count (which allocates) on two
calls in a row; results are integers, so they must be equal.  This file is
collected last on purpose; it passes alone in a fresh process and after the
other tests."""
import ctypes
import random

import pytest

pytestmark = pytest.mark.gpu


def _records(seed, n, n_keys, n_graphs):
    r = random.Random(seed)
    keys = [r.randrange(n_keys) for _ in range(n)]
    gids = sorted(r.randrange(n_graphs) for _ in range(n))
    return keys, gids


def _call_noalloc(gs, torch, keys, gids, n_keys, n_graphs, out):
    dk = torch.tensor(keys, dtype=torch.int32, device="cuda")
    dg = torch.tensor(gids, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = gs.lib().gs_support_count_noalloc(ctypes.c_void_p(dk.data_ptr()), ctypes.c_void_p(dg.data_ptr()),
                                           len(keys), n_keys, n_graphs, ctypes.c_void_p(out.data_ptr()),
                                           ctypes.c_void_p(stream))
    assert st == 0, gs.lib().gs_last_error()
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


def test_noalloc_rejects_oversized_bitmaps(gs):
    torch = pytest.importorskip("torch")
    out = torch.zeros(1 << 12, dtype=torch.int32, device="cuda")
    # 4096 keys x 8192 words (262,144 graphs) > 1,048,576 words
    st = gs.lib().gs_support_count_noalloc(None, None, 0, 1 << 12, 1 << 18, ctypes.c_void_p(out.data_ptr()), None)
    assert st == 8  # GS_ERR_LIMIT
    assert b"exceeds" in gs.lib().gs_last_error()
