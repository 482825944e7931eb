"""The committed ncu summaries that bench.py reads: the step kernel's DRAM
traffic per launch for each storage format at 256^3 parses, and lies within 5%
of the algorithmic bytes (26 distributions read and written: 208 B/node FP32,
108 B/node with 16-bit storage and an FP32 f_0), i.e. no re-reads."""
from __future__ import annotations

import pytest

ALG = {"fp32": 208, "fp16": 108, "bf16": 108}


@pytest.mark.parametrize("storage", sorted(ALG))
def test_step_traffic_summary_matches_the_algorithmic_bytes(storage):
    import bench
    traffic = bench.profiled_traffic(storage, 256)
    assert traffic is not None, f"profiles/zsc_step_{storage}_256cube.txt has no dram_bytes_per_launch line"
    alg = ALG[storage] * 256 ** 3
    assert 0.95 <= traffic / alg <= 1.05, traffic / alg
    assert bench.BYTES_PER_NODE[storage] == ALG[storage]
