"""q-point sharding across processes (one per GPU, no data exchange), run as
two gloo ranks on the CPU: the shards of rp_calc_chiqw (rp_plan_q) and of
bench.py are disjoint and together cover every q point still to do."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, root: str, out_dir: str):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from respackdev_gb300 import chiqw as rp

        nl = ("&param_chiqw\n Ecut_for_eps=3.0, Green_func_delt=0.2721 /\n"
              f"&param_gpu\n qshard_index={rank}, qshard_count={world} /\n")
        mine = rp.plan_q(root, nl)
        bmine = bench.shard_q(8, rank, world)
        got = [None] * world
        dist.all_gather_object(got, (mine, bmine))
        if rank == 0:
            with open(os.path.join(out_dir, "shards.txt"), "w") as f:
                f.write(repr(got))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _run(root, out_dir, world=2):
    mp.spawn(_worker, args=(world, _free_port(), root, out_dir), nprocs=world, join=True)
    with open(os.path.join(out_dir, "shards.txt")) as f:
        return eval(f.read())


def test_q_shards_are_disjoint_and_complete(case_dir, fresh_copy, tmp_path):
    root = fresh_copy(case_dir("tiny"))
    got = _run(root, str(tmp_path))
    lib = [set(g[0]) for g in got]
    assert lib[0].isdisjoint(lib[1])
    assert lib[0] | lib[1] == set(range(1, 9))
    assert abs(len(lib[0]) - len(lib[1])) <= 1
    b = [set(g[1]) for g in got]
    assert b[0].isdisjoint(b[1]) and b[0] | b[1] == set(range(2, 9))


def test_q_shards_skip_finished_points(case_dir, fresh_copy, tmp_path):
    """q points whose dat.log.400 exists (an earlier, interrupted run) are left
    out of every shard (chiqw.F:593-608)."""
    root = fresh_copy(case_dir("tiny"))
    for iq in (3, 5):
        d = os.path.join(root, "dir-eps", "q%03d" % iq)
        os.makedirs(d, exist_ok=True)
        open(os.path.join(d, "dat.log.400"), "w").close()
    got = _run(root, str(tmp_path))
    lib = [set(g[0]) for g in got]
    assert lib[0].isdisjoint(lib[1])
    assert lib[0] | lib[1] == {1, 2, 4, 6, 7, 8}
