"""Root-subtree partitioning across processes (one GPU each).

The DFS-code tree below each frequent 1-edge code is independent of the
others: the reference's root loop (src/gspan_cuda/gspan_cuda_no_sort.cpp:
90-124, src/gspan/gspan.cpp:300-330) mines them one after another with no
shared state.  Rank r of n mines the frequent roots whose index, in the
reference's root order, is r modulo n (gs_mine_opts.root_part/root_parts),
with the whole database resident on its own GPU.  No data is exchanged while
mining; the only communication is gathering the pattern lists at the end,
and merging them restores the single-process output order exactly: the
k-th root group of rank r is root k*n + r.
"""


def root_groups(patterns, is_root=None):
    """Splits a traversal-ordered pattern list into its root groups (each
    starts with a 1-edge pattern, followed by that root's subtree)."""
    if is_root is None:
        def is_root(p):
            return len(p[0]) == 1
    groups = []
    for p in patterns:
        if is_root(p) or not groups:
            groups.append([])
        groups[-1].append(p)
    return groups


def merge_root_partitions(parts, is_root=None):
    """parts[r] = the patterns rank r mined with root_part=r, root_parts=len(parts);
    returns the patterns in the order one process mining every root emits."""
    groups = [root_groups(p, is_root) for p in parts]
    n = len(parts)
    out = []
    k = 0
    while True:
        took = False
        for r in range(n):
            if k < len(groups[r]):
                out.extend(groups[r][k])
                took = True
        if not took:
            return out
        k += 1


def mine_partitioned(db, minsup, group=None, miner=None, **kw):
    """Mines this rank's share of the root subtrees and gathers every rank's
    patterns (torch.distributed, any backend; a default group must exist).

    Returns the merged list on every rank.  `miner(db, minsup, root_part,
    root_parts, **kw)` returns this rank's [(code, support)] in traversal
    order; it defaults to gpu_graph_mining_gb300.mine_collect."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    if miner is None:
        from . import mine_collect

        def miner(d, s, root_part, root_parts, **k2):
            pats, _ = mine_collect(d, s, root_part=root_part, root_parts=root_parts, **k2)
            return pats
    local = miner(db, minsup, rank, world, **kw)
    if world == 1:
        return local
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    return merge_root_partitions(parts)
