"""CPU checks of the serving loop's host logic: the admission rule, the
memory estimate it uses, and argument checking without a GPU."""
import ctypes

import numpy as np
import pytest

from libgwmodel_gb300 import _lib


def admit(budget, reserved, busy, estimate):
    n = len(reserved)
    r = (ctypes.c_double * n)(*reserved)
    b = (ctypes.c_int * n)(*busy)
    return _lib.lib().gwgpu_admit_slot(float(budget), n, r, b, float(estimate))


def test_admits_into_a_free_slot_within_budget():
    assert admit(100, [0, 0, 0], [0, 0, 0], 10) in (0, 1, 2)
    assert admit(100, [50, 0, 0], [1, 0, 0], 10) in (1, 2)


def test_prefers_a_slot_that_already_holds_enough():
    # slot 2 holds 30 >= 20: no growth; slot 1 holds 25 (smaller, still enough) wins
    assert admit(100, [40, 25, 30], [1, 0, 0], 20) == 1
    # nobody holds enough: grow the one holding most
    assert admit(100, [5, 8, 3], [0, 0, 0], 20) == 1


def test_waits_when_every_slot_is_busy():
    assert admit(100, [10, 10], [1, 1], 1) == -1


def test_waits_when_the_budget_would_be_exceeded():
    # running requests hold 90; growing the idle slot to 20 would need 110
    assert admit(100, [45, 45, 0], [1, 1, 0], 20) == -1
    # the idle slot's own memory counts: growing 15 -> 20 keeps 95 <= 100
    assert admit(100, [40, 40, 15], [1, 1, 0], 20) == 2


def test_estimate_grows_with_the_problem():
    L = _lib.lib()
    e = lambda n, p, g, prec, a: L.gwgpu_estimate_bytes(n, p, g, prec, a)
    base = e(10000, 5, 0, 0, 1)
    assert base > 8 * 10000 * 5
    assert e(20000, 5, 0, 0, 1) > base
    assert e(10000, 10, 0, 0, 1) > base
    assert e(10000, 5, 0, 1, 1) > base      # the mixed path adds its tensor-core images
    assert e(10000, 5, 1, 0, 1) > base      # geographic keeps radians and caps
    assert e(10000, 5, 0, 0, 0) < base      # no histogram cache or order statistics without adaptive
    # config-4 extreme: n = 100,000, p = 20, well below a 150 GB budget even for 16 slots
    assert 16 * e(100000, 20, 1, 1, 1) < 150e9


def test_server_needs_a_device():
    L = _lib.lib()
    count = ctypes.c_int(-1)
    rc = L.gwgpu_device_count(ctypes.byref(count))
    if rc == _lib.OK and count.value > 0:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert L.gwgpu_server_create(0, 1e9, 2, ctypes.byref(h)) != _lib.OK
    assert L.gwgpu_server_create(0, 1e9, 0, ctypes.byref(h)) == _lib.ERR_INVALID
    assert L.gwgpu_server_submit(None, None, None, None) == _lib.ERR_INVALID
