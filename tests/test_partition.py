"""Root-subtree partitioning across ranks: gloo on CPU, world size 2 and 3.
Each rank mines its share with the oracle standing in for its GPU (the
partition rule is the same: frequent roots in the reference's order, index
modulo the number of parts); the product's merge must give back the
single-process output, in order."""
import os
import socket

import pytest

from conftest import GOLDEN, REPO, read_lines, run_oracle


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, oracle, path, minsup, out):
    import sys
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    from gpu_graph_mining_gb300.partition import mine_partitioned
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def miner(db, s, root_part, root_parts):
        lines = run_oracle(oracle, "txt", db, s, ["--roots", "%d/%d" % (root_part, root_parts)])
        return [(tuple(l.split("\t")[0].split(";")), int(l.split("\t")[1])) for l in lines]
    merged = mine_partitioned(path, minsup, miner=miner)
    if rank == 0:
        with open(out, "w") as f:
            f.write("\n".join("%s\t%d" % (";".join(c), s) for c, s in merged) + "\n")
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_root_partition_merge_gloo(oracle, tmp_path, world):
    import torch.multiprocessing as mp
    path = os.path.join(GOLDEN, "cfg1_seed1.txt")
    out = str(tmp_path / "merged.txt")
    mp.start_processes(_worker, args=(world, _free_port(), oracle, path, 10, out), nprocs=world,
                       start_method="spawn")
    assert read_lines(out) == run_oracle(oracle, "txt", path, 10)


def test_merge_round_robin():
    from gpu_graph_mining_gb300.partition import merge_root_partitions
    r = lambda n: ((0,),) * n  # noqa: E731  code with n edges
    a = [(r(1), "A0"), (r(2), "A0x"), (r(1), "A2")]
    b = [(r(1), "B1"), (r(1), "B3"), (r(3), "B3x")]
    got = [s for _, s in merge_root_partitions([a, b])]
    assert got == ["A0", "A0x", "B1", "A2", "B3", "B3x"]
