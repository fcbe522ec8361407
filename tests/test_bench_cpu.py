"""The bench's contract on the CPU: the reference arm's JSON line, the
algorithmic byte count it reports the roofline with, and the rule that a
DRAM traffic figure is reported only for the kernel sources it was captured
on."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_algorithmic_bytes_per_substep():
    assert bench.BYTES_PER_SUBSTEP == sum(bench.STAGE_BYTES.values()) == 753
    assert bench.STAGE_BYTES["density"] == 36


def test_traffic_only_for_the_captured_sources(monkeypatch):
    digest = bench.csrc_digest(bench.KERNEL_SOURCES["density"])
    monkeypatch.setattr(bench, "NCU_TRAFFIC", {"density": (1.0e8, digest)})
    traffic, source = bench.roofline_traffic("density", "plain_large")
    assert traffic == 1.0e8 and digest in source
    monkeypatch.setattr(bench, "NCU_TRAFFIC", {"density": (1.0e8, "0" * 12)})
    assert bench.roofline_traffic("density", "plain_large")[0] is None
    assert bench.roofline_traffic("density", "column")[0] is None
    assert bench.roofline_traffic("sort", "plain_large")[0] is None


def test_digest_depends_on_the_named_sources_only():
    a = bench.csrc_digest(["sf_kernels.cu"])
    assert a == bench.csrc_digest(["sf_kernels.cu"])
    assert a != bench.csrc_digest(["sf_sort.cu"])
    assert len(bench.csrc_digest()) == 12


@pytest.mark.timeout(600)
def test_reference_arm_json_line():
    """`bench.py --impl reference`: the FP32 restatement of the reference
    kernels on the host cores, one JSON line with the driver's keys."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["metric"] == "particle-substeps/s at 1M SPH+DEM" and line["unit"] == "particle-substeps/s"
    assert line["config"]["workload"] == "plain_large" and line["config"]["particles"] > 1_000_000
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
