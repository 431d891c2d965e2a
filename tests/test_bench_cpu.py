"""The benchmark's result-line contract (host side, no GPU): every required key is checked
before the line is printed, and the reference arm (the CPU restatement on the host cores) runs
and prints one line of the same metric."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.conftest import ROOT


def _line():
    return {"metric": "m", "value": 1.0, "unit": "runs/s", "n_gpus": 1, "steps": 3, "warmup": 3, "ms_per_step": 1.0,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "w"}, "gpu_launches": 3,
            "roofline": {"bound": "fp32", "achieved": 1.0, "peak": 2.0, "unit": "TFLOP/s", "frac": 0.5, "traffic": None},
            "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []},
            "e2e": {"value": 1.0, "unit": "runs/s", "h2d_bytes_per_step": 8, "d2h_bytes_per_step": 8},
            "cpu_baseline": {"value": 0.1, "unit": "runs/s", "cores": 8, "kind": "port", "sample": "s"}}


def test_complete_line_passes():
    import bench
    assert bench.check_line(_line()) is not None


@pytest.mark.parametrize("path", ["value", "roofline", "e2e", "cpu_baseline", "gpu_launches", "clocks",
                                  "roofline.traffic", "e2e.d2h_bytes_per_step", "cpu_baseline.kind",
                                  "clocks.reasons", "config.workload"])
def test_missing_key_raises(path):
    import bench
    line = _line()
    parent, _, leaf = path.rpartition(".")
    del (line[parent] if parent else line)[leaf]
    with pytest.raises(RuntimeError, match="lacks"):
        bench.check_line(line)


def test_switched_off_parts_are_not_required():
    import bench
    line = _line()
    del line["e2e"], line["cpu_baseline"]
    bench.check_line(line, e2e=False, cpu=False)


def test_reference_arm_prints_one_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "runs/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def test_plain_sample_is_stratified_by_dimension():
    """The plain single-run comparison times one run per equal-width stratum of D, weighted by
    the stratum's run count (a run's cost grows steeply with D); a single-dimension batch gives
    evenly spaced runs of equal weight."""
    import bench
    wl = bench.workload(4096, 2024, "config3")
    Ds = np.array([w[0] for w in wl])
    idx, weight = bench.plain_sample(Ds)
    assert len(idx) == 8 and sum(weight) == len(wl)
    edges = np.linspace(Ds.min(), Ds.max() + 1, 9)
    for k, (r, wt) in enumerate(zip(idx, weight)):
        assert edges[k] <= Ds[r] < edges[k + 1]
        assert wt == np.count_nonzero((Ds >= edges[k]) & (Ds < edges[k + 1]))
    assert min(Ds[idx]) <= 8 and max(Ds[idx]) >= 58  # the sample reaches both ends of D
    idx, weight = bench.plain_sample(np.full(1024, 10))
    assert idx == list(range(0, 1024, 128)) and weight == [128.0] * 8
