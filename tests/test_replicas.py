"""The N > 1 bench path on CPU: two gloo ranks run the replica aggregation the bench uses
under torchrun; both see the slowest rank's time and the whole-job body-steps/s."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist

    from nbody_gb300.replicas import whole_job_value

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank          # rank 1 is slower
    value, max_ms, w = whole_job_value(local_ms, bodies_per_rank=1000, steps=10)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(f"{value} {max_ms} {w}")


def test_two_gloo_ranks_agree_on_the_slowest(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    results = [tuple(map(float, (tmp_path / f"r{r}.txt").read_text().split())) for r in range(2)]
    assert results[0] == results[1]
    value, max_ms, world = results[0]
    assert world == 2 and max_ms == 150.0
    assert value == pytest.approx(1000 * 10 * 2 / 0.150)


def test_single_process_value():
    from nbody_gb300.replicas import whole_job_value
    value, max_ms, world = whole_job_value(200.0, 4096, 5)
    assert world == 1 and max_ms == 200.0 and value == pytest.approx(4096 * 5 / 0.2)
