"""bench_bal, the drop-in CLI (reference benchmarks/bench_bal.cpp:4-134): flags,
exit codes and the JSON schema. Argument and IO errors (exit 1) need no GPU;
solves are GPU tests."""
import json
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "gpu-bundle-adjustment_gb300" / "bin" / "bench_bal"
TINY = ROOT / "tests" / "golden" / "tiny_problem.txt"

# the reference's keys, in its order (bench_bal.cpp:104-123)
REFERENCE_KEYS = ["file", "solver", "loss", "num_cameras", "num_points", "num_observations", "initial_cost",
                  "final_cost", "iterations", "total_time_s", "per_iteration_s", "termination", "device"]


def _run(*args, timeout=120):
    return subprocess.run([str(BIN), *map(str, args)], capture_output=True, text=True, timeout=timeout)


@pytest.fixture(scope="module", autouse=True)
def _built(gba):  # the gba fixture builds the library and bench_bal
    if not BIN.exists():
        pytest.skip("bench_bal not built")


@pytest.mark.parametrize("args", [
    [],                                            # no problem
    ["--iterations=x", str(TINY)],                 # bad value
    ["--frobnicate", str(TINY)],                   # unknown flag
    [str(TINY), "--synthetic=1"],                  # both inputs
    [str(TINY), "--loss=cauchy"],                  # unknown loss (bench_ceres.cpp:138-141)
    [str(TINY), "--loss=huber", "--delta=0"],      # Huber needs delta > 0
    ["/nonexistent/problem.txt"],                  # unreadable file
])
def test_argument_and_io_errors_exit_1(args):
    r = _run(*args)
    assert r.returncode == 1, (r.returncode, r.stderr)


@pytest.mark.gpu
def test_json_schema_and_file_output(tmp_path):
    out = tmp_path / "r.json"
    r = _run(TINY, "--iterations=5", f"--json={out}")
    assert r.returncode == 0, r.stderr
    printed = json.loads(r.stdout)
    assert list(printed)[:len(REFERENCE_KEYS)] == REFERENCE_KEYS
    assert json.loads(out.read_text()) == printed
    assert printed["num_cameras"] == 5 and printed["num_points"] == 300 and printed["num_observations"] == 882
    assert printed["loss"] == "none"
    assert printed["termination"] in ("CONVERGENCE", "MAX_ITERATIONS")
    assert printed["final_cost"] < printed["initial_cost"]
    assert printed["trajectory"][0] == printed["initial_cost"]


MODEL = ROOT / "gpu-bundle-adjustment_gb300" / "models" / "coarse_mlp.bin"


@pytest.mark.gpu
@pytest.mark.parametrize("extra", [["--form=mixed"], ["--form=mixed", "--refine-tol=0.1", "--pcg-tol=0.1"],
                                   ["--loss=huber", "--delta=2"], ["--form=mixed", "--loss=huber", "--delta=2"],
                                   ["--form=learned", f"--model={MODEL}"]])
def test_forms_and_loss(extra):
    r = _run(TINY, "--iterations=10", *extra)
    assert r.returncode == 0, r.stderr
    j = json.loads(r.stdout)
    assert j["loss"] == ("huber" if "--loss=huber" in extra else "none")
    assert j["final_cost"] < j["initial_cost"]


@pytest.mark.gpu
def test_non_finite_observation_exits_3(tmp_path):
    """A non-finite observation: the device anomaly counter moves and bench_bal
    refuses to report (exit 3, reference bench_bal.cpp:95-99)."""
    lines = TINY.read_text().splitlines()
    parts = lines[1].split()
    parts[2] = "nan"
    lines[1] = " ".join(parts)
    bad = tmp_path / "nan.txt"
    bad.write_text("\n".join(lines) + "\n")
    r = _run(bad, "--iterations=3")
    assert r.returncode == 3, (r.returncode, r.stderr)
