"""Multi-GPU runs are replicas: every rank runs the whole workload on its own
GPU and only the timing is combined (maximum over ranks).  These tests run
that host logic as two gloo ranks on the CPU under torchrun, the way the
benchmark is launched for N > 1."""
import json
import os
import socket
import subprocess
import sys
import textwrap

from conftest import ROOT


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, cwd, timeout=240):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=cwd, env=env, capture_output=True, text=True, timeout=timeout)


def test_reduce_max_and_barrier_two_gloo_ranks(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent(f"""
        import json, os, sys
        sys.path.insert(0, {str(ROOT)!r})
        import torch.distributed as dist
        import bench
        dist.init_process_group("gloo")
        rank, world = dist.get_rank(), dist.get_world_size()
        bench.barrier(world)
        m = bench.reduce_max(1.5 + 10.0 * rank, world)
        bench.barrier(world)
        with open(os.path.join({str(tmp_path)!r}, f"rank{{rank}}.json"), "w") as f:
            json.dump({{"rank": rank, "world": world, "max": m}}, f)
        dist.destroy_process_group()
    """))
    r = torchrun([str(script)], cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-2000:]
    got = [json.loads((tmp_path / f"rank{k}.json").read_text()) for k in range(2)]
    assert [g["world"] for g in got] == [2, 2]
    assert [g["max"] for g in got] == [11.5, 11.5]


def test_reference_arm_under_torchrun_prints_once(trove_lib):
    """--impl reference at N = 2: rank 0 alone runs the CPU port and prints one
    line; rank 1 exits 0 without work."""
    import oracle
    oracle.lib()  # built before the ranks start
    r = torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--workload", "gather", "--steps", "1",
                  "--warmup", "0"], cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_clock_sampler_without_a_gpu():
    """The timed region's clock record degrades to a reasoned null when
    neither NVML nor nvidia-smi can be opened (as on a machine without a
    GPU), instead of failing the run."""
    import torch
    sys.path.insert(0, str(ROOT))
    import bench
    c = bench.clock_sampler(torch, torch.device("cuda", 0))
    rec = c.stop()
    assert set(rec) >= {"sm_mhz", "sm_max_mhz", "reasons"}
    if rec.get("source") == "nvml":  # a machine with a GPU: real samples
        assert rec["samples"] >= 1 and rec["sm_mhz"] > 0
    elif rec["sm_mhz"] is None:
        assert rec["reasons"] == ["nvidia-smi unavailable"] or rec.get("samples") == 0
