"""The multi-rank path of bench.py on CPU: two gloo ranks run the same
bookkeeping the GPU ranks run over NCCL (join, barrier, slowest-rank time,
whole-job rate), and the reference arm reports from rank 0 only."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as td

    import bench
    r, w, local = bench.dist()
    bench.init_ranks(w, local, backend="gloo")
    bench.barrier(w)
    ms = 100.0 + 50.0 * r  # rank 1 is the slow one
    m = bench.max_over_ranks(ms, w, device="cpu")
    v = bench.job_rate(6, w, m * 1e-3)
    bench.barrier(w)
    td.destroy_process_group()
    q.put((r, m, v))


def test_two_gloo_ranks_agree_on_the_slowest_time():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in procs)
    assert [r for r, _, _ in res] == [0, 1]
    for _, m, v in res:
        assert m == 150.0
        assert v == pytest.approx(6 * 2 / 0.150)


def _args(**kw):
    import argparse
    a = argparse.Namespace(gpus=2, steps=3, warmup=3, impl="reference", res=64, hires=128,
                           cg_accuracy=1e-4, blur_type=1, e2e_steps=2, no_cpu_baseline=False)
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def test_reference_arm_reports_from_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    class FakeCpu:
        def __init__(self, R, H, acc):
            assert (R, H) == (64, 128)
            self.parts = {"solves_s": 3.0}

        def step(self):
            return 4.0

    monkeypatch.setattr(bench, "CpuWorkload", FakeCpu)
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    bench.run_reference(_args())
    assert capsys.readouterr().out == ""
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("LOCAL_RANK", "0")
    bench.run_reference(_args())
    out = capsys.readouterr().out.strip().splitlines()
    assert len(out) == 1
    line = json.loads(out[0])
    assert line["impl"] == "reference"
    assert line["value"] == pytest.approx(2.0 / 4.0)  # two solves per whole step
    # one whole step, reported as run (the driver's step counts ask for more)
    assert line["steps"] == 1 and line["warmup"] == 0 and line["ms_per_step"] == 4000.0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"] == bench.flof_config(_args(), 2)
    assert line["metric"] == bench.METRIC and line["higher_is_better"] is True


def test_step_hbm_and_network_flops():
    sys.path.insert(0, ROOT)
    import bench
    recs = [("cg_matvec", 64, 1.0e9, 0.2), ("gauss_blur", 64, 2.0e9, 1.0)]
    h = bench.step_hbm(recs, 2, 100.0, 6800.0, "measured")
    assert h["bytes_per_step"] == 1.5e9
    assert h["achieved"] == pytest.approx(1.5e9 / 0.05 / 1e9, rel=1e-3)
    assert h["frac"] == pytest.approx(h["achieved"] / 6800.0, abs=1e-4)  # rounded to 4 places
    # 2 * taps * cin * cout per output voxel and layer; training = forward,
    # weight gradients and the input gradients of every layer but the first
    R = 16
    fwd = (2 * 81 * (2 * 16 * R ** 4 + 16 * 32 * (R // 2) ** 4 + 32 * 32 * (R // 2) ** 4
                     + 32 * 64 * (R // 4) ** 4 + 64 * 64 * (R // 4) ** 4 + 96 * 32 * (R // 2) ** 4
                     + 48 * 16 * R ** 4) + 2 * 16 * 4 * R ** 4)
    assert bench.net_flops(R) == fwd
    assert bench.net_train_flops(R) == 3 * fwd - 2 * 81 * 2 * 16 * R ** 4
