"""The reference's segmented scan and reduction (src/reduction) as GPU single
operators, pinned by the reference's own tests:
  * src/reduction/tests/scan_test.cpp:8-90: every element 1, a segment head
    every `segment_size` elements; inclusive and exclusive scans against a
    host running sum, at the test's shapes (1024 x 32, 1000 x 10, 505 x
    10..24, 16/15/17 x 10..249);
  * src/reduction/tests/reduction_test.cpp:9-70 (the same shapes reduced:
    every segment sums to its size, or size - 1 exclusive) and its
    multi-segment shapes (:150-190);
  * src/reduction/tests/reduction_test_bugs.cpp:12-40 (a 60-element vector
    with literal results 9, 1, 1, 4, 2, 10);
  * src/reduction/tests/reduction_test_bug2.cpp:13-80 (276 segments of 12
    with a random number of leading ones each).
The host restatement `_host_scan` is checked against the literal vector on
the CPU; the GPU results are compared with it."""
import random

import pytest

HEAD = 0x80000000

# reduction_test_bugs.cpp:13-18
BUG1 = [1, 0, 1, 1, 1, 1, 1, 1, 1, 1,
        2147483648, 1, 0, 0, 0, 0, 0, 0, 0, 0,
        2147483648, 1, 0, 0, 0, 0, 0, 0, 0, 0,
        2147483648, 1, 1, 0, 0, 0, 0, 1, 1, 0,
        2147483648, 0, 1, 0, 1, 0, 0, 0, 0, 0,
        2147483649, 1, 1, 1, 1, 1, 1, 1, 1, 1]
BUG1_RESULT = [9, 1, 1, 4, 2, 10]


def _host_scan(data, exclusive):
    """Running sum of bits 0-30 that restarts at every bit-31 flag (element 0
    starts a segment), modulo 2^32: the check in scan_test.cpp:40-60."""
    out, run = [], 0
    for i, x in enumerate(data):
        v = x & 0x7fffffff
        if i == 0 or x & HEAD:
            run = 0
        run = (run + v) & 0xffffffff
        out.append((run - v) & 0xffffffff if exclusive else run)
    return out


def _host_reduce(data, counts, sizes, exclusive):
    s = _host_scan(data, exclusive)
    ends, at = [], 0
    for c, z in zip(counts, sizes):
        for _ in range(c):
            at += z
            ends.append(at - 1)
    return [s[e] for e in ends]


def _uniform(segment_size, segment_count):
    # scan_test.cpp:14-22 / reduction_test.cpp:14-22
    return [1 | (HEAD if i % segment_size == 0 and i != 0 else 0) for i in range(segment_size * segment_count)]


def _multi(sizes, counts):
    # reduction_test.cpp:86-110: heads every size within a run of segments
    n = sum(s * c for s, c in zip(sizes, counts))
    out, idx, cnt, start = [], 0, 0, 0
    for i in range(n):
        v = 1
        if (i - start) % sizes[idx] == 0 and i != 0:
            v |= HEAD
            cnt += 1
            if cnt == counts[idx]:
                cnt, idx, start = 0, idx + 1, i
        out.append(v)
    return out


def _bug2(block_size, block_count, seed):
    # reduction_test_bug2.cpp:13-45: each block starts with rand() % block_size ones
    r = random.Random(seed)
    data, want = [], []
    ones = r.randrange(block_size)
    want.append(ones)
    for i in range(block_size * block_count):
        v = 0
        if i > 0 and i % block_size == 0:
            v += HEAD
            ones = r.randrange(block_size)
            want.append(ones)
        if ones > 0:
            v += 1
            ones -= 1
        data.append(v)
    return data, want


SHAPES = [(1024, 32), (1000, 10)] + [(505, i) for i in range(10, 25, 7)] + \
         [(z, i) for z in (16, 15, 17) for i in (10, 11, 63, 64, 65, 128, 249)]


def test_host_restatement_matches_literal_vector():
    assert _host_reduce(BUG1, [6], [10], False) == BUG1_RESULT
    d, want = _bug2(12, 276, 3)
    assert _host_reduce(d, [276], [12], False) == want


@pytest.mark.gpu
@pytest.mark.parametrize("exclusive", [False, True])
def test_segmented_scan_shapes(gs, exclusive):
    for size, count in SHAPES:
        d = _uniform(size, count)
        assert gs.segmented_scan(d, exclusive) == _host_scan(d, exclusive), (size, count)


@pytest.mark.gpu
@pytest.mark.parametrize("exclusive", [False, True])
def test_segmented_reduce_shapes(gs, exclusive):
    for size, count in SHAPES:
        got = gs.segmented_reduce(_uniform(size, count), [count], [size], exclusive)
        assert got == [size - 1 if exclusive else size] * count, (size, count)
    for sizes, counts in [([30, 50], [10, 15]), ([30, 50, 32, 52, 42], [10, 15, 10, 15, 15]),
                          ([14, 16, 18, 50, 100], [5, 40, 5, 40, 50]), ([15, 16, 32, 50, 32], [8, 8, 16, 32, 33]),
                          ([100, 1000, 100, 2000, 10], [20, 20, 20, 20, 20])]:
        got = gs.segmented_reduce(_multi(sizes, counts), counts, sizes, exclusive)
        want = [z - 1 if exclusive else z for z, c in zip(sizes, counts) for _ in range(c)]
        assert got == want, sizes


@pytest.mark.gpu
def test_segmented_reduce_bug_vectors(gs):
    assert gs.segmented_reduce(BUG1, [6], [10]) == BUG1_RESULT
    for seed in range(4):
        d, want = _bug2(12, 276, seed)
        assert gs.segmented_reduce(d, [276], [12]) == want


@pytest.mark.gpu
def test_segmented_scan_random(gs):
    r = random.Random(9)
    for n in [0, 1, 2, 1023, 1024, 1025, 70000, 1 << 20]:
        d = [r.randrange(1 << 31) | (HEAD if r.random() < 0.01 else 0) for _ in range(n)]
        for ex in (False, True):
            assert gs.segmented_scan(d, ex) == _host_scan(d, ex), n
    # no heads at all: one segment, sums wrap modulo 2^32
    d = [0x7fffffff] * 5000
    assert gs.segmented_scan(d) == _host_scan(d, False)
    with pytest.raises(gs.GSpanError):
        gs.segmented_reduce([1, 2, 3], [2], [2])  # segments run past the array
