"""The real-data fixture (tests/golden/realdata.npz) against the reference's
MAT files it was extracted from (when the reference checkout is present),
and the scan constants utilities/test_asdpocs.m hard-codes against the ones
stored in swine_2d.mat."""
import os
import sys

import numpy as np
import pytest

from conftest import REFERENCE as REF
from conftest import ROOT, golden


def test_swine_constants_match_driver():
    d = golden("realdata.npz")
    sod, sdd, dt = d["swine_geo"]
    # test_asdpocs.m: dt = 0.148, sod = 405.9410, sdd = 906.2510
    assert (sod, sdd, dt) == (405.9410, 906.2510, 0.148)
    assert d["swine_P"].shape == (1537, 90) and d["head190"].shape == (512, 512)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "testdata")),
                    reason="reference test data not present")
def test_fixture_is_the_reference_data():
    pytest.importorskip("scipy")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_realdata

    fresh = make_realdata.extract(REF)
    d = golden("realdata.npz")
    for k, v in fresh.items():
        assert np.array_equal(d[k], v), k
