"""bench.py's multi-rank host logic on the CPU (gloo, world size 2, on
127.0.0.1): the step time reported by rank 0 is the maximum over the ranks'
replicas, and the reference arm runs on rank 0 only (the other ranks return
without work or output)."""
import importlib.util
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = _bench().max_over_ranks(values[rank], world)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    values = [0.147, 0.162]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert out[0] == out[1] == 0.162


def test_single_rank_is_identity():
    assert _bench().max_over_ranks(0.25, 1) == 0.25


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    bench = _bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "cpu_full_run", lambda *a, **k: called.append(1))

    class Args:
        steps, warmup, gpus = 1, 0, 2

    assert bench.run_reference(Args()) is None
    assert not called and capsys.readouterr().out == ""


def test_reference_arm_json_contract():
    """bench.py --impl reference prints one JSON line with the keys of the
    bench contract (metric, value, unit, timing, config, cpu_baseline, e2e),
    here on CAS(6e,6o) so that a full run takes about a second: the value is
    the mean of full CPU runs (no extrapolation), each one's time listed."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--norb", "6", "--nel", "6", "--nchol", "12"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["n_gpus"] == 1 and line["steps"] == 1
    assert line["higher_is_better"] is False and line["value"] > 0
    assert abs(line["ms_per_step"] - line["value"] * 1e3) < 1e-6 * line["ms_per_step"]
    cb, e2e = line["cpu_baseline"], line["e2e"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert cb["sample"].startswith("full") and cb["runs"] == 1 and cb["run_values"] == [line["value"]]
    assert cb["iterations"] > 0 and cb["energy"] < 0
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"]
