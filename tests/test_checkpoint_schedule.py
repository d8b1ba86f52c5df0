"""The binomial checkpoint schedule of the checkpointed adjoint (host code,
no GPU): it reverses every step once, stores no more states than it has
slots for, and recomputes no more forward steps than the optimum, which a
brute-force recursion gives here for small cases (Griewank & Walther,
ACM TOMS 26(1), 2000: fewest forward steps to reverse l steps with c
checkpoints)."""
import ctypes
import functools
import os

import pytest

from geophyinv_gb300 import _build, _lib


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_build.LIB):
        _build.build()
    return _lib.load()


@functools.lru_cache(maxsize=None)
def optimum(n, c):
    """Fewest advances (turn steps not counted) to reverse n steps with c
    checkpoints, one holding the start."""
    if n <= 1:
        return 0
    if c <= 1:
        return n * (n - 1) // 2
    return min(m + optimum(n - m, c - 1) + optimum(m, c) for m in range(1, n))


def schedule(lib, nt, slots):
    adv, turns, stored = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
    assert lib.gpi_checkpoint_schedule(nt, slots, ctypes.byref(adv), ctypes.byref(turns), ctypes.byref(stored)) == 0
    return adv.value, turns.value, stored.value


@pytest.mark.parametrize("slots", [1, 2, 3, 5])
def test_schedule_is_optimal_for_small_cases(lib, slots):
    for nt in range(1, 41):
        adv, turns, stored = schedule(lib, nt, slots)
        assert turns == nt
        assert stored <= slots
        # the forward_save run makes the first sweep's advances; the adjoint
        # run makes the rest
        first = optimum(nt, slots + 1)
        assert adv <= first, (nt, slots, adv, first)


def test_schedule_at_workload_sizes(lib):
    # 3000 steps with 30 slots (a checkpoint every 100 steps): about two
    # recomputations of each step at most
    adv, turns, stored = schedule(lib, 3000, 30)
    assert turns == 3000 and stored == 30
    assert adv < 3 * 3000
    adv2, _, _ = schedule(lib, 3000, 300)
    assert adv2 < adv
    # fewer slots, more recomputation
    assert schedule(lib, 200, 1)[0] > schedule(lib, 200, 5)[0] > schedule(lib, 200, 50)[0]


def test_schedule_rejects_bad_arguments(lib):
    assert lib.gpi_checkpoint_schedule(0, 3, None, None, None) != 0
    assert lib.gpi_checkpoint_schedule(10, 0, None, None, None) != 0
