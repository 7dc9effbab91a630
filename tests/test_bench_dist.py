"""Multi-process plumbing of bench.py on CPU (gloo, world size 2): the
max-over-ranks timing and the reference arm's rank-0-only run. The solve path
itself runs as independent replicas (no collective on the data path)."""
import importlib.util
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _load_bench()
        out[rank] = bench.max_over_ranks(1.5 + rank, world, device="cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    torch = pytest.importorskip("torch")
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_rank_max_is_identity():
    bench = _load_bench()
    assert bench.max_over_ranks(3.25, 1) == 3.25


def test_reference_arm_only_on_rank0(monkeypatch, capsys):
    bench = _load_bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = bench.argparse.Namespace(workload=1, seed=None, reference_iterations=1, warmup=0, steps=1)
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""


def test_clock_summary_keeps_the_timed_window():
    """The clock summary uses the samples inside the timed window; with fewer
    than two there, it adds the nearest sample on either side."""
    import datetime as dt

    bench = _load_bench()
    t = dt.datetime(2026, 1, 1, 12, 0, 0)
    ms = lambda k: t + dt.timedelta(milliseconds=k)
    row = lambda mhz, cap="Not Active": [str(mhz), "2070", "Not Active", "Not Active", "Not Active", cap]

    s = bench.ClockSampler()
    s.samples = [(ms(0), row(900)), (ms(100), row(2070)), (ms(200), row(2060, "Active")), (ms(300), row(800))]
    s.window = (ms(50), ms(250))
    out = s.summary()
    assert out["samples_in_window"] == 2 and out["samples_used"] == 2
    assert out["sm_mhz"] == 2065 and out["sm_max_mhz"] == 2070 and out["reasons"] == ["sw_power_cap"]

    s.window = (ms(120), ms(180))  # no sample inside: bracket with the neighbours
    out = s.summary()
    assert out["samples_in_window"] == 0 and out["samples_used"] == 2 and out["sm_mhz"] == 2065

    s.window = None
    assert s.summary()["reasons"] == ["unsampled"]


def test_clock_sampler_devices_follow_the_ranks(monkeypatch):
    """Rank r runs on visible device r mod count; nvidia-smi gets the physical
    identifiers (CUDA_VISIBLE_DEVICES entries when set)."""
    bench = _load_bench()
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    assert bench.smi_devices(1, 8) == ["0"]
    assert bench.smi_devices(4, 8) == ["0", "1", "2", "3"]
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "3, 5")
    assert bench.smi_devices(2, 2) == ["3", "5"]
    assert bench.smi_devices(1, 2) == ["3"]
    assert bench.ClockSampler(["3", "5"]).devices == "3,5"


def _run_bench(*argv):
    import json
    import subprocess

    code = ("import sys, runpy; sys.argv = ['bench.py'] + sys.argv[1:]; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "print('LOADED', 'gba_gb300' in sys.modules)")
    r = subprocess.run([sys.executable, "-c", code, *argv], cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env={**os.environ, "RANK": "0", "WORLD_SIZE": "1"})
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    return json.loads(lines[-2]), lines[-1]


def test_reference_arm_samples_workload5_without_the_library():
    """Workload 5 is too large for whole CPU solves: each step is a bounded
    sample (normal equations over every observation + a Cholesky at n = 4,608
    scaled to 45,000), reported as an extrapolated lower bound."""
    line, loaded = _run_bench("--impl", "reference", "--steps", "1", "--warmup", "0")
    assert loaded == "LOADED False"
    assert line["impl"] == "reference" and "unavailable" not in line
    assert line["unit"] == "s" and line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["iterations_to_target"] == 8
    assert line["cpu_baseline"]["extrapolated"] and line["cpu_baseline"]["kind"] == "port"
    assert "8788960 observations" in line["cpu_baseline"]["sample"]


def test_reference_arm_times_oracle_solves_to_target_workload1():
    line, loaded = _run_bench("--impl", "reference", "--workload", "1", "--steps", "1", "--warmup", "0")
    assert loaded == "LOADED False"  # the CPU arm never loads the product library
    assert line["impl"] == "reference" and line["unit"] == "s" and line["value"] > 0
    assert line["config"]["iterations_to_target"] is not None
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
