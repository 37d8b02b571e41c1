"""The C++ API mirror run on the GPU: nscale::imreconstruct / imfillHoles / bwlabel2 /
bwareaopen2 / imhmin and nscale::gpu::imreconstruct / imreconstructQueueThroughput /
boundingBox2, nscale::morphOpen and nscale::distanceTransform give the oracle's
results; a type mismatch raises cv::Exception."""
import subprocess

import numpy as np
import pytest

from cpp_api import build

pytestmark = pytest.mark.gpu


def test_cpp_api_matches_oracle(nsgb, oracle, tmp_path):
    exe = tmp_path / "nscale_api_test"
    build(str(exe))
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    H, W = 300, 400

    def load(name, dt):
        return np.fromfile(tmp_path / name, dtype=dt).reshape(H, W)

    mask, marker = load("mask.u8", np.uint8), load("marker.u8", np.uint8)
    rec8 = oracle.imreconstruct(marker, mask, 8)
    assert np.array_equal(load("recon8.u8", np.uint8), rec8)
    assert np.array_equal(load("recon4.u8", np.uint8), oracle.imreconstruct(marker, mask, 4))
    assert np.array_equal(load("batch0.u8", np.uint8), rec8)
    assert np.array_equal(load("batch1.u8", np.uint8), rec8)
    assert np.array_equal(load("speedup8.u8", np.uint8), rec8)
    bin_dark = np.where(mask < 128, 255, 0).astype(np.uint8)
    assert np.array_equal(load("speedup_bin8.u8", np.uint8),
                          oracle.imreconstruct_binary(load("bseed.u8", np.uint8), bin_dark, 8))
    fill = oracle.imfill_holes(oracle.threshold_gt(rec8, 128.0), True, 4)
    assert np.array_equal(load("fill4.u8", np.uint8), fill)
    lab, _ = oracle.bwlabel2(fill, 8, True)
    assert np.array_equal(load("labels8.i32", np.int32), lab)
    flat, count = oracle.bwareaopen2(fill, False, True, 11, 1000, 8)
    assert np.array_equal(load("area.u8", np.uint8), flat)
    assert f"count {count} " in r.stdout
    assert np.array_equal(load("hmin8.u8", np.uint8), oracle.imhmin(mask, 10, 8))
    cross = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], np.uint8)
    assert np.array_equal(load("open3.u8", np.uint8), oracle.morph_open(mask, cross))
    bin_mask = np.where(mask < 128, 255, 0).astype(np.uint8)
    assert np.array_equal(load("dist.f32", np.float32), oracle.distance_transform(bin_mask))
    box = oracle.bounding_box(lab, 0)
    assert f"boxes {box.shape[1]}" in r.stdout
    assert np.array_equal(np.fromfile(tmp_path / "bbox.i32", dtype=np.int32).reshape(5, -1), box)
