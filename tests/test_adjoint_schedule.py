"""The adjoint's binomial checkpointing schedule (host logic, no GPU):
lbm_adjoint_forward_steps runs the same recursion as lbm_step_adjoint without
stepping.  Checked against the exact optimum of that recursion (dynamic
programming over the first checkpoint, terminal state included) on small cases,
and against Griewank's minimum r T - beta(n + 1, r - 1) (n snapshots, r the
smallest sweep count with beta(n, r) >= T) on the benchmark's cases."""
from __future__ import annotations

from math import comb

import pytest


def beta(n, r):
    return comb(n + r, r)


def exact_optimum(L, C):
    """u[l][c]: fewest forward steps to reverse the last l steps of the run (the
    terminal state still to build) from a stored start with c free slots."""
    t = [[0] * (C + 1) for _ in range(L + 1)]
    u = [[0] * (C + 1) for _ in range(L + 1)]
    for l in range(1, L + 1):
        t[l][0] = l * (l - 1) // 2
        u[l][0] = 1 if l == 1 else l + l * (l - 1) // 2
    for c in range(1, C + 1):
        u[1][c] = 1
        for l in range(2, L + 1):
            t[l][c] = min(m + t[l - m][c - 1] + t[m][c] for m in range(1, l))
            u[l][c] = min(m + u[l - m][c - 1] + t[m][c] for m in range(1, l))
    return u


def test_schedule_is_within_one_step_of_the_exact_optimum(lib):
    from lbm_bench_gpu_gb300 import capi
    L, C = 80, 6
    u = exact_optimum(L, C)
    for slots in range(2, C + 2):
        for T in range(2, L + 1):
            got = capi.adjoint_forward_steps(T, slots)
            opt = u[T][min(slots, T + 1) - 1]
            assert opt <= got <= opt + 1, (T, slots, got, opt)


@pytest.mark.parametrize("T,slots", [(2000, 183), (2000, 677), (20000, 44), (300, 18), (5000, 10)])
def test_schedule_reaches_griewank_minimum(lib, T, slots):
    from lbm_bench_gpu_gb300 import capi
    r = 1
    while beta(slots, r) < T:
        r += 1
    minimum = r * T - beta(slots + 1, r - 1) + 1   # + the terminal state
    got = capi.adjoint_forward_steps(T, slots)
    assert minimum <= got <= minimum + 8, (got, minimum)


def test_schedule_edge_cases(lib):
    from lbm_bench_gpu_gb300 import capi
    assert capi.adjoint_forward_steps(20, 21) == 20      # a slot per state: one sweep
    assert capi.adjoint_forward_steps(20, 500) == 20     # more slots than states
    assert capi.adjoint_forward_steps(1, 1) == 1
    assert capi.adjoint_forward_steps(10, 1) == 10 + 45  # no free slot: recompute from the start
    assert capi.adjoint_forward_steps(0, 5) == -1 and capi.adjoint_forward_steps(5, 0) == -1


def test_two_tier_schedule_counts():
    """lbm_adjoint_forward_steps_tiers: the forward steps of the schedule with a
    second tier of host checkpoints.  The long-horizon case (20 000 steps, 44
    device slots, 66 host slots) is the count a GB300 run of lbm_step_adjoint
    reported; no host slots is the one-tier count; host slots never add
    forward steps there, and fewer device slots never take fewer."""
    from lbm_bench_gpu_gb300 import capi
    assert capi.adjoint_forward_steps(20000, 44, 66) == 56774
    assert capi.load().lbm_adjoint_forward_steps_tiers(20000, 44, 0) == capi.adjoint_forward_steps(20000, 44)
    assert capi.adjoint_forward_steps(20000, 44, 66) < capi.adjoint_forward_steps(20000, 44)
    assert capi.adjoint_forward_steps(20, 3, 4) == 38 and capi.adjoint_forward_steps(20, 5, 4) == 33
    for slots in (4, 8, 16):
        assert capi.adjoint_forward_steps(2000, slots, 30) >= capi.adjoint_forward_steps(2000, slots + 1, 30)
    assert capi.load().lbm_adjoint_forward_steps_tiers(0, 4, 3) == -1
