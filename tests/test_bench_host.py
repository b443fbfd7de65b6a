"""bench.py's reference arm (the oracle's restatement of big-wave's slice-step on the host cores)
keeps its JSON contract, and ranks other than 0 exit without work. A 256^2 case keeps it short."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def run(env_extra=None):
    env = {**os.environ, **(env_extra or {})}
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "256", "--steps", "1",
                           "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)


def test_reference_arm_json_line():
    r = run()
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "slice-steps/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["vs_baseline"] is None and line["n_gpus"] == 1
    assert (line["steps"], line["warmup"]) == (1, 1) and line["ms_per_step"] > 0
    assert line["config"]["workload"] == "talbot_lau_256x256_c64"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_do_nothing():
    r = run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_pass_kernel_names_follow_the_schedule_rules():
    """The kernels the bench line names for each pass: split pairs where they exist, the dithered
    one-per-group kernels where they are the only dithered form (rows of 16384 and 3*2^k, columns
    of 3*2^k), the compensated kernels under bits 16 / 32."""
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.pass_kernels(64, 4096) == {"row_pass": "row_pass_kernel", "col_pass": "col_x2_pipe_kernel"}
    assert bench.pass_kernels(0, 4096) == {"row_pass": "row_x2_kernel", "col_pass": "col_x2_pipe_kernel"}
    assert bench.pass_kernels(192, 4096) == {"row_pass": "row_pass_kernel", "col_pass": "col_pipe_kernel"}
    assert bench.pass_kernels(0, 3072) == {"row_pass": "row_pass_kernel", "col_pass": "col_pipe_kernel"}
    assert bench.pass_kernels(48, 3072) == {"row_pass": "row_pass_kernel", "col_pass": "col_pass_kernel"}
    assert bench.pass_kernels(51, 3072) == {"row_pass": "row_pipe_kernel", "col_pass": "col_pipe_kernel"}
    assert bench.pass_kernels(0, 16384)["row_pass"] == "row_pass_kernel"
    assert bench.schedule_name(0, 3072) == "rows:dithered-single,cols:dithered-single"
    assert bench.schedule_name(64, 4096) == "rows:dithered-single,cols:split-pair"
    assert bench.schedule_name(48, 3072) == "rows:per-block-voxel,cols:per-block"
    assert bench.schedule_name(16, 16384) == "rows:per-block-voxel,cols:per-block"
    assert bench.schedule_name(8, 16384) == "rows:dithered-single,cols:split-3-pass (last slice per-block)"
    assert bench.schedule_name(42, 4096) == "rows:split-pair,cols:split-3-pass (last slice pipelined)"
