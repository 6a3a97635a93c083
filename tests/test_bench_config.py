"""The bench's workloads are the reference's measured configurations: the
2D sparse-view head-slice protocol (the headline), the 3D cone-beam volume,
the batched uneven slices and the serving stream, with their sizes, views,
bins, distances, noise and iteration counts."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, ROOT)
    import bench as b

    return b


def test_headline_fan_beam_protocol(bench, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    args, W = bench.parse()
    assert args.workload == "fan2d" and args.gpus == 1 and args.warmup >= 3
    assert (W["nx"], W["ny"], W["nz"]) == (512, 512, 1)
    assert (W["nv"], W["na"], W["nb"], W["det"]) == (60, 888, 1, 1.0)
    assert (W["SO"], W["SO"] + W["OD"]) == (541.0, 949.0)
    assert (W["I0"], W["iters"], W["ng"], W["batch"]) == (1e5, 100, 20, 64)
    assert W["phantom"] == "ellipses"


def test_cone_beam_volume(bench, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "cone3d"])
    _, W = bench.parse()
    assert (W["nx"], W["ny"], W["nz"], W["vx"]) == (256, 256, 256, 1.0)
    assert (W["nv"], W["na"], W["nb"], W["det"]) == (360, 512, 512, 0.8)
    assert (W["SO"], W["SO"] + W["OD"]) == (1000.0, 1500.0)
    assert (W["I0"], W["iters"], W["phantom"]) == (5e4, 50, "shepp_logan")


def test_uneven_slices_and_serving_stream(bench, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "uneven"])
    _, W = bench.parse()
    assert W["batch"] == 64
    assert W["sizes"] == (256, 384, 512, 768) and W["views"] == (60, 120, 360, 720)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "serve"])
    _, W = bench.parse()
    assert (W["rate"], W["frac2d"]) == (20.0, 0.7)
