"""bench.py --impl reference on the host CPU: the reference's own kernels
(compiled for the CPU from its sources) time a box of the workload, and the
JSON line carries what the driver reads from it: impl "reference", the metric
and unit of the GPU arm, a cpu_baseline describing the run, an e2e object with
no host-device bytes, and the GPU arm's config when the whole box ran."""
from __future__ import annotations

import json

import pytest

from oracle.oracle import ref_lib

pytestmark = pytest.mark.skipif(ref_lib() is None, reason="reference sources not staged")


def test_reference_arm_json_line(capsys):
    import bench
    argv = ["--impl", "reference", "--steps", "1", "--warmup", "1", "--size", "64", "--bubbles", "4"]
    assert bench.main(argv) == 0
    d = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "MLUPS" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "reference" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the whole 64^3 box ran, so the config is the one the GPU arm reports for these arguments
    args = bench.parse_args(argv)
    assert d["config"] == bench.workload_config(args, bench.workload(64, 4), 1)
