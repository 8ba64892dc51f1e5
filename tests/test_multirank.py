"""The N>1 path of bench.py on CPU: two gloo ranks (one process per GPU in a
real run) share no data-path collective; only the timing aggregation crosses
ranks.  Whole-job throughput is all ranks' converged solves over the slowest
rank's step, and the reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.dist_barrier(w)
    # rank 1 is the slower one; each rank converged a different count per step
    dev_ms = [[100.0, 110.0], [150.0, 170.0]][rank]
    wall_s = [[0.2, 0.2], [0.3, 0.5]][rank]
    conv = [[219, 219], [218, 220]][rank]
    step_s, e2e_s, converged, value, e2e_value = bench.aggregate_ranks(w, dev_ms, wall_s, conv)
    # the reference arm: ranks other than 0 exit without work
    ran_reference = bench.run_reference(None, w, r) if r != 0 else None
    out[rank] = (step_s, e2e_s, converged, value, e2e_value, ran_reference)
    import torch.distributed as dist
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_gloo_ranks_aggregate_max_and_sum():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
    assert set(out.keys()) == {0, 1}
    for rank in (0, 1):
        step_s, e2e_s, converged, value, e2e_value, ran_ref = out[rank]
        assert step_s == pytest.approx(0.160)          # max of the ranks' mean device steps
        assert e2e_s == pytest.approx(0.4)            # max of the mean end-to-end steps
        assert converged == pytest.approx(438.0)      # 219 + 219 converged solves per step
        assert value == pytest.approx(438.0 / 0.160)
        assert e2e_value == pytest.approx(438.0 / 0.4)
    assert out[1][5] is None


@pytest.mark.parametrize("env,local,expect", [
    ({}, 3, "3"),                                        # nothing exported: the local rank
    ({"CUDA_VISIBLE_DEVICES": "0,1,2,3,4,5,6,7"}, 5, "5"),  # one list for every rank: its entry
    ({"CUDA_VISIBLE_DEVICES": "4,5,6,7"}, 2, "6"),
    ({"CUDA_VISIBLE_DEVICES": "6"}, 6, "6"),              # already one device per rank: kept
    ({"CUDA_VISIBLE_DEVICES": "GPU-aa,GPU-bb"}, 1, "GPU-bb"),
])
def test_each_rank_gets_its_own_gpu(env, local, expect):
    """One process per GPU: each rank restricts itself to its own device
    before its first CUDA call, whatever list the launcher exported."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_device_env(local, env) == expect


def test_clocks_sampled_on_the_rank_gpu(monkeypatch):
    """The clock sampler watches the GPU the process computes on."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    assert bench.sampled_gpu(2) == "2"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "5")
    assert bench.sampled_gpu(0) == "5"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "3,4")
    assert bench.sampled_gpu(0) == "3"
