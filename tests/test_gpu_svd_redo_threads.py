"""The fallback of the batched dense sigma (matrices the fast kernel could not finish
are redone by the FP64-polished Jacobi kernel) is per call and per host thread: two
host threads going through it at once get the polished results, and the
process-wide "svd_fast" switch is unchanged afterwards."""
import ctypes
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _opt(C, name):
    v = ctypes.c_int(-1)
    C.check(C.lib().hbem_get_option(name.encode(), ctypes.byref(v)))
    return v.value


def test_redo_in_two_threads_keeps_the_switch():
    from helmholtzbem_gb300 import _capi as C, api, geometry

    ks = np.linspace(1.0, 6.0, 7)

    def ops():
        return [api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 12), order=7)),
                api.SolutionsOperator(api.BuilderData(geometry.polygon(*geometry.star_polygon(8, 5), 14),
                                                      order=7))]

    fast = api.sweep_sigma_multi(ops(), [ks, ks], 1.0, [5.0, 3.0], d=2)
    assert _opt(C, "svd_fast") == 1
    # what the fallback computes: the polished kernel's results
    C.check(C.lib().hbem_set_option(b"svd_fast", 0))
    try:
        polished = api.sweep_sigma_multi(ops(), [ks, ks], 1.0, [5.0, 3.0], d=2)
    finally:
        C.check(C.lib().hbem_set_option(b"svd_fast", 1))
    C.check(C.lib().hbem_set_option(b"svd_fast_force_redo", 1))
    try:
        out, errs = [None, None], []

        def run(t):
            try:
                mine = ops()
                for _ in range(3):
                    out[t] = api.sweep_sigma_multi(mine, [ks, ks], 1.0, [5.0, 3.0], d=2)
            except Exception as ex:   # reported by the main thread
                errs.append(ex)

        th = [threading.Thread(target=run, args=(t,)) for t in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errs, errs
    finally:
        C.check(C.lib().hbem_set_option(b"svd_fast_force_redo", 0))
    assert _opt(C, "svd_fast") == 1 and _opt(C, "svd_fast_force_redo") == 0
    for got in out:   # both threads went through the fallback: the polished kernel's values
        for a, b in zip(got, polished):
            np.testing.assert_array_equal(a, b)
    # and the fast kernel is still the one a later sweep takes
    again = api.sweep_sigma_multi(ops(), [ks, ks], 1.0, [5.0, 3.0], d=2)
    for a, b in zip(again, fast):
        np.testing.assert_array_equal(a, b)
