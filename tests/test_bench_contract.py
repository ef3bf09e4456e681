"""The bench's reference arm on the CPU: one JSON line with the metric
contract's keys (the GPU arm is run on a GB300, not here), timed on the
oracle alone -- no library of the product is mapped into the process."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

PROBE = """
import sys
sys.argv = ["bench.py", "--impl", "reference", "--config", "0", "--steps", "2", "--warmup", "0",
            "--ref-fp64-steps", "1"]
sys.path.insert(0, {root!r})
import bench
rc = bench.main()
maps = open("/proc/self/maps").read()
print("PRODUCT_LIB_MAPPED" if "libswap_gpu" in maps else "ORACLE_ONLY", "liboracle" in maps)
sys.exit(rc)
"""


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "-c", PROBE.format(root=str(ROOT))], capture_output=True, text=True,
                       timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["dtype"] == "f32" and d["fp64"]["precision"] == "f64" and d["fp64"]["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"]
    # every timed step is a full step of the whole workload
    assert d["config"]["ions"] == 64 * 32 * 32 * 16 and d["warmup"] == 3 and len(d["step_s"]) == 2
    assert abs(d["ms_per_step"] - 1e3 * sum(d["step_s"]) / 2) <= 0.01 * d["ms_per_step"] + 2
    tail = r.stdout.strip().splitlines()[-1].split()
    assert tail == ["ORACLE_ONLY", "True"], tail


def test_reference_arm_under_torchrun_prints_one_line():
    """Launched as the multi-GPU bench is (torchrun, two ranks on 127.0.0.1),
    the reference arm runs on rank 0 alone and prints one line; the other
    rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29611", str(ROOT / "bench.py"), "--impl", "reference",
           "--config", "0", "--steps", "1", "--warmup", "0", "--ref-fp64-steps", "0", "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
