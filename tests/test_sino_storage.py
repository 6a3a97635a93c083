"""Host rounding of sinograms to FP16 / BF16 storage (asdpocs_store_sinogram,
the bits the plans and the serving queue keep on the device): round to
nearest with ties to even, checked against numpy's float16 conversion and
against an independent nearest-value search for BF16."""
import ctypes as C

import numpy as np
import pytest

from asd_pocs_mex_cuda_demo_gb300._lib import SINO_STORAGE, AsdpocsError, check


def _store(lib, x, fmt):
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros(x.size, np.uint16 if fmt != "f32" else np.float32)
    check(lib.asdpocs_store_sinogram(x.ctypes.data, out.ctypes.data, x.size,
                                     SINO_STORAGE[fmt]))
    return out


def _values():
    rng = np.random.default_rng(4)
    parts = [
        rng.standard_normal(20000) * 10.0 ** rng.uniform(-9, 6, 20000),
        # every float near the FP16 subnormal / normal / overflow boundaries
        np.float32(2.0 ** -24) * np.arange(-70, 70),
        np.array([6.1e-5, 6.09e-5, 2 ** -14, 65504, 65519.99, 65520, 65536, 1e30, -1e30,
                  0.0, -0.0, np.inf, -np.inf, 2 ** -25, 1.5 * 2 ** -25, 3 * 2 ** -26]),
        # ties: values exactly halfway between FP16 / BF16 neighbours
        (1 + (2 * np.arange(1, 200) + 1) * 2.0 ** -11) * 2.0 ** rng.integers(-10, 10, 199),
        (1 + (2 * np.arange(1, 200) + 1) * 2.0 ** -8) * 2.0 ** rng.integers(-60, 60, 199),
    ]
    return np.concatenate(parts).astype(np.float32)


def test_fp16_storage_rounds_like_ieee(lib):
    x = _values()
    got = _store(lib, x, "f16")
    with np.errstate(over="ignore"):  # values past 65504 round to inf, as intended
        want = x.astype(np.float16).view(np.uint16)
    assert np.array_equal(got, want)


def _bf16_nearest(x):
    """BF16 of each FP32 by picking the nearer of the two neighbouring BF16
    values in double precision, the even one on a tie."""
    bits = x.view(np.uint32).astype(np.uint64)
    lo = (bits >> 16).astype(np.uint32)
    hi = lo + 1

    def val(h):
        return (h.astype(np.uint32) << 16).view(np.float32).astype(np.float64)

    xv = x.astype(np.float64)
    dlo, dhi = np.abs(xv - val(lo)), np.abs(val(hi) - xv)
    pick_hi = (dhi < dlo) | ((dhi == dlo) & ((lo & 1) == 1))
    out = np.where(pick_hi, hi, lo).astype(np.uint16)
    exact = (bits & 0xFFFF) == 0
    return np.where(exact, lo.astype(np.uint16), out)


def test_bf16_storage_rounds_to_nearest_even(lib):
    x = _values()
    x = x[np.isfinite(x) & (np.abs(x) < 3.0e38)]
    got = _store(lib, x, "bf16")
    assert np.array_equal(got, _bf16_nearest(x))


def test_storage_of_non_finite_values(lib):
    x = np.array([np.nan, -np.nan, np.inf, -np.inf], np.float32)
    for fmt, dt in (("f16", np.float16), ("bf16", None)):
        got = _store(lib, x, fmt)
        if dt is not None:
            v = got.view(np.float16).astype(np.float32)
        else:
            v = (got.astype(np.uint32) << 16).view(np.float32)
        assert np.isnan(v[:2]).all() and v[2] == np.inf and v[3] == -np.inf


def test_fp32_storage_is_a_copy_and_bad_storage_is_refused(lib):
    x = _values()
    assert np.array_equal(_store(lib, x, "f32").view(np.uint32), x.view(np.uint32))
    out = np.zeros(4, np.uint16)
    with pytest.raises(AsdpocsError, match="unknown sinogram storage"):
        check(lib.asdpocs_store_sinogram(x.ctypes.data, out.ctypes.data, 4, 7))
