"""Extract the real-data fixture (tests/golden/realdata.npz) from the
reference's test data (testdata/*.mat, MATLAB v5 files), read with scipy.

Run where the reference checkout exists:

    python tests/golden/make_realdata.py [reference root]

Stored:
* ``swine_P`` -- the 90 columns of ``prjSwine`` (1537 bins x 360 one-degree
  views of a swine scan) that utilities/test_asdpocs.m reconstructs: views
  4, 8, ..., 360 degrees (MATLAB columns (1:90)*4; the script as written
  indexes (1:360)*4, past the 360 columns of the file, so the 90-view reading
  is the one that runs), float32;
* ``swine_geo`` -- sod, sdd and detector pitch stored in the file;
* ``head190`` -- the 512 x 512 uint16 slice of P10240000_head_slice190.mat
  that demo_head190.m uses as its phantom.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def extract(ref_root):
    import scipy.io as sio

    td = os.path.join(ref_root, "testdata")
    sw = sio.loadmat(os.path.join(td, "swine_2d.mat"))
    cols = np.arange(1, 91) * 4 - 1  # MATLAB columns (1:90)*4, 0-based
    P = np.asarray(sw["prjSwine"], np.float64)[:, cols].astype(np.float32)
    geo = np.array([float(sw["sod"].ravel()[0]), float(sw["sdd"].ravel()[0]),
                    float(sw["detPixelSize"].ravel()[0])])
    head = sio.loadmat(os.path.join(td, "P10240000_head_slice190.mat"))["img_slice190"]
    return dict(swine_P=P, swine_geo=geo, head190=np.asarray(head, np.uint16))


if __name__ == "__main__":
    # the reference checkout: an argument, ASDPOCS_REFERENCE_DIR, else a
    # checkout named "reference" beside the repository
    root = (sys.argv[1] if len(sys.argv) > 1
            else os.environ.get("ASDPOCS_REFERENCE_DIR")
            or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))),
                            "reference"))
    np.savez_compressed(os.path.join(HERE, "realdata.npz"), **extract(root))
