"""Write-step sums: the host half (no GPU).

``pp_pairwise_plan`` writes the summation tree of NumPy's float64 sum; the
plan, followed on the host (``writes.evaluate_plan``), must give
``np.sum`` bit for bit on every length, which pins the order the device
kernel follows.  Also the tip-list layout and the argument checks of
``pp_write_sums`` that run before any CUDA call.
"""
import ctypes

import numpy as np
import pytest

SIZES = (list(range(0, 40)) + [63, 64, 65, 127, 128, 129, 130, 136, 255, 256,
                               257, 1000, 4095, 8192, 8193, 12_345, 65_537,
                               200_003])


@pytest.fixture(scope="module")
def L():
    from probabilistic_peridynamics_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        from probabilistic_peridynamics_gb300 import build
        build.build()
    return _lib.lib()


@pytest.mark.parametrize("n", SIZES)
def test_plan_reproduces_numpy_sum(n, L):
    from probabilistic_peridynamics_gb300.writes import (evaluate_plan,
                                                         pairwise_plan)
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n) * 10.0 ** rng.integers(-8, 8, size=n)
    plan = pairwise_plan(n)
    assert plan[3] == n
    assert evaluate_plan(plan, a) == np.sum(a)
    # the products the reference sums: force * volume[:, None], (n, 3)
    if n % 3 == 0 and n:
        f = a.reshape(-1, 3)
        vol = rng.uniform(0.5, 2.0, size=n // 3) * 1e-6
        assert evaluate_plan(plan, (f * vol[:, None]).ravel()) == \
            np.sum(f * vol[:, np.newaxis])


def test_plan_shape(L):
    from probabilistic_peridynamics_gb300.writes import pairwise_plan
    p = pairwise_plan(1_200_000)
    leaves, inner, heights = int(p[0]), int(p[1]), int(p[2])
    assert inner == leaves - 1
    lens = p[4 + leaves:4 + 2 * leaves]
    assert lens.sum() == 1_200_000 and lens.min() >= 64 and lens.max() <= 128
    los = p[4:4 + leaves]
    assert np.array_equal(los[1:], np.cumsum(lens)[:-1])
    off = p[4 + 2 * leaves + 2 * inner:]
    assert off.size == heights + 1 and off[0] == 0 and off[-1] == inner
    # children precede parents: every child index is below its parent's
    left = p[4 + 2 * leaves:4 + 2 * leaves + inner]
    right = p[4 + 2 * leaves + inner:4 + 2 * leaves + 2 * inner]
    parent = leaves + np.arange(inner)
    assert np.all(left < parent) and np.all(right < parent)
    assert pairwise_plan(0)[:4].tolist() == [0, 0, 0, 0]
    assert pairwise_plan(5)[:4].tolist() == [1, 0, 0, 5]


def test_signed_zeros_and_non_finite(L):
    from probabilistic_peridynamics_gb300.writes import (evaluate_plan,
                                                         pairwise_plan)
    for a in (np.full(300, -0.0), np.full(5, -0.0),
              np.array([1.0, np.inf, -1.0] * 50),
              np.array([np.inf, -np.inf] + [1.0] * 200)):
        with np.errstate(invalid="ignore"):
            got = evaluate_plan(pairwise_plan(a.size), a)
            want = np.sum(a)
        assert (got == want and np.signbit(got) == np.signbit(want)) or \
            (np.isnan(got) and np.isnan(want))


def test_plan_rejects_bad_lengths(L):
    from probabilistic_peridynamics_gb300.writes import pairwise_plan
    with pytest.raises(ValueError):
        pairwise_plan(-1)
    with pytest.raises(ValueError):
        pairwise_plan(2 ** 31)
    # too small a buffer: the length comes back, nothing is written
    buf = np.full(4, 7, dtype=np.int32)
    need = L.pp_pairwise_plan(1000, buf.ctypes.data_as(ctypes.c_void_p), 4)
    assert need > 4 and np.all(buf == 7)


def test_tip_entries_follow_dict_order():
    from probabilistic_peridynamics_gb300.writes import tip_entries
    offsets, entries = tip_entries({"3": [(5, 0), (9, 2)], "1": [],
                                    "deflection": [(0, 1)]})
    assert offsets.tolist() == [0, 2, 2, 3]
    assert entries.tolist() == [[5, 0], [9, 2], [0, 1]]
    offsets, entries = tip_entries({})
    assert offsets.tolist() == [0] and entries.shape == (0, 2)


def test_write_sums_validation_without_gpu(L):
    from probabilistic_peridynamics_gb300 import _lib
    a = _lib.WriteSumsArgs()
    assert L.pp_write_sums(None, None) == _lib.PP_ERROR_INVALID_VALUE
    a.nnodes = 10
    assert L.pp_write_sums(ctypes.byref(a), None) == \
        _lib.PP_ERROR_INVALID_VALUE  # NULL arrays
    a.nnodes = 2 ** 30
    assert L.pp_write_sums(ctypes.byref(a), None) == _lib.PP_ERROR_TOO_LARGE
    a.nnodes, a.ntips = 10, -1
    assert L.pp_write_sums(ctypes.byref(a), None) == \
        _lib.PP_ERROR_INVALID_VALUE
