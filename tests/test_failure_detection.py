"""Failure detection without a GPU fault: the only device-side wait (the sort's look-back) is made to wait on a flag
that nothing sets; it gives up after its poll limit, records ASPH_DEVERR_SPIN_LIMIT in the error word, and the
context stays usable. Host-side failures (bad arguments, budget) are covered by the C-ABI and server tests."""
import ctypes
import time

import pytest

from adaptivesph_gb300 import _lib
from helpers import assert_state_bitexact, make_pair, small_dam_break

pytestmark = pytest.mark.gpu

SPIN_LIMIT = 0x1


def test_bounded_wait_runs_out_and_reports():
    L = _lib.load()
    word = ctypes.c_uint32(0)
    t = time.perf_counter()
    _lib.check(L.asph_debug_wait_limit_probe(ctypes.byref(word)), "asph_debug_wait_limit_probe")
    assert word.value & SPIN_LIMIT, word.value
    assert time.perf_counter() - t < 60.0
    # the context is still usable: a small simulation steps bit-exactly afterwards
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    for _ in range(3):
        sim.update(sc.dt)
        orc.step(sc.dt)
    assert_state_bitexact(sim.read_state(), orc.arrays())
    assert sim.device_errors() == 0
