"""bench.py on CPU: the constants it reads from the committed ncu summaries
(instructions per processed face for the issue roofline, DRAM bytes per
launch for the HBM roofline) parse and agree with the counts the summaries
state, and the reference arm prints one JSON line with the keys of the
measurement contract."""
import json
import os
import re
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def _first(pattern, text):
    m = re.search(pattern, text)
    assert m, pattern
    return m


@pytest.mark.parametrize("workload", ["batch", "waves"])
def test_instructions_per_face_match_the_stated_counts(workload):
    """The per-face figure is the first capture's smsp__inst_executed.sum
    over the processed faces of its case."""
    ipf = bench.profile_instructions(workload)
    assert ipf is not None and 1.0 < ipf < 50.0
    text = open(os.path.join(REPO, "profiles", f"chunk_kernel_{workload}.txt")).read()
    block = text[:text.index("warp_instructions_per_processed_face:")]
    inst = float(list(re.finditer(r"smsp__inst_executed\.sum ([0-9.]+) M", block))[-1].group(1)) * 1e6
    faces = float(list(re.finditer(r"processed faces of the case ([0-9.]+) M", block))[-1].group(1)) * 1e6
    assert inst / faces == pytest.approx(ipf, rel=2e-3)
    # only one line carries the key, so bench.py cannot pick up an older count
    assert text.count("warp_instructions_per_processed_face:") == 1


def test_traffic_per_launch_scales_the_stated_capture():
    """DRAM bytes of a full config-1 launch: the capture's read + write bytes
    scaled by processed faces (27.97 M in the full launch)."""
    traffic = bench.profile_traffic("batch")
    assert traffic is not None
    text = open(os.path.join(REPO, "profiles", "chunk_kernel_batch.txt")).read()
    assert text.count("dram_bytes_per_full_launch:") == 1
    m = _first(r"DRAM traffic per processed face: ([0-9.]+) MB / ([0-9.]+) M", text)
    per_face = float(m.group(1)) / float(m.group(2))
    assert traffic == pytest.approx(per_face * 1e6 * 27.97, rel=5e-3)
    # the capture's own read + write lines add up to the stated total
    rd = float(_first(r"dram__bytes_read\.sum\s+([0-9.]+) MB", text).group(1))
    wr = float(_first(r"dram__bytes_write\.sum\s+([0-9.]+) MB", text).group(1))
    assert rd + wr == pytest.approx(float(m.group(1)), abs=0.02)


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "3"], cwd=REPO, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["config"]["workload"] == "mixed_batch_4096_bodies_distinct_meshes"
    assert d["value"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_under_torchrun_prints_once():
    """Launched as the multi-GPU runs are (torchrun, two ranks), rank 0 alone
    runs the reference arm and prints its line; the other rank exits 0."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                          "--master-addr", "127.0.0.1", "--master-port", str(port),
                          os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "3"], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
