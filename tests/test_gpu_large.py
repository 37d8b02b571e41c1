"""The large single-image workload: 16384 x 16384 (268 Mpixel) with about 102k ellipses,
hole filling by reconstruction by erosion (marker = image on the border, max elsewhere) in
4- and 8-connectivity, threshold > 128 (scaled with the dtype) and bwlabel (8-connected,
raster relabel) of the result, all device-resident; plus bwlabel of the dark objects
(image <= 128: about 69k components, the 102k ellipses minus the overlapping ones).

Every stage is compared with the reference's own imfillHoles<T> / `Mat > k` / bwlabel2 on the
same image, through the SHA-256 digests of their outputs in tests/golden/ref_recon_digests.json
(i32 under the saturating CV_32S reading of invert<int>(INT_MIN)); where a digest is absent,
with the oracle."""
import json
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def image_u8():
    import workloads as W

    return W.c4("u8")


@pytest.fixture(scope="module")
def c4_digests():
    d = json.load(open(os.path.join(ROOT, "tests", "golden", "ref_recon_digests.json")))
    return d.get("c4")


def _oracle_stage(oracle, img, conn, thr):
    fill = oracle.imfill_holes(img, False, conn)
    b = oracle.threshold_gt(fill, thr)
    lab, n = oracle.bwlabel2(b, 8, True)
    return fill, lab, n


@pytest.mark.parametrize("dtype", ["u8", "u16", "i32"])
def test_large_fill_threshold_label(nsgb, oracle, image_u8, c4_digests, dtype):
    import torch

    import workloads as W
    from nsgb import synth

    img = image_u8 if dtype == "u8" else synth.scale(image_u8, dtype)[0]
    thr = 128.0 * W.SCALE[dtype]
    d_img = torch.from_numpy(img).cuda()
    got = {}
    for conn in (4, 8):
        fill = nsgb.imfillHoles(d_img, False, conn)
        b = nsgb.threshold(fill, thr)
        lab, n = nsgb.bwlabel2_count(b, 8)
        got[conn] = (fill.cpu().numpy(), lab.cpu().numpy(), n)
        del fill, b, lab
    # dark objects: the complement of (image > thr)
    dk = nsgb.invert(nsgb.threshold(d_img, thr))
    dlab, dn = nsgb.bwlabel2_count(dk, 8)
    dlab = dlab.cpu().numpy()
    assert dn > 50000
    if c4_digests is not None:
        for conn in (4, 8):
            exp = c4_digests[f"{dtype}_conn{conn}"]
            fill_g, lab_g, n_g = got[conn]
            assert W.digest(fill_g) == exp["fill"], f"fill conn={conn}"
            assert n_g == exp["n_labels"] and W.digest(lab_g) == exp["labels"], f"labels conn={conn}"
        exp = c4_digests[f"{dtype}_dark"]
        assert dn == exp["n_labels"] and W.digest(dlab) == exp["labels"]
        return
    with ThreadPoolExecutor(3) as ex:
        futs = {conn: ex.submit(_oracle_stage, oracle, img, conn, thr) for conn in (4, 8)}
        dark = ex.submit(lambda: oracle.bwlabel2(255 - oracle.threshold_gt(img, thr), 8, True))
        for conn in (4, 8):
            fill_e, lab_e, n_e = futs[conn].result()
            fill_g, lab_g, n_g = got[conn]
            assert np.array_equal(fill_g, fill_e), f"fill conn={conn}"
            assert n_g == n_e and np.array_equal(lab_g, lab_e), f"labels conn={conn}"
        dlab_e, dn_e = dark.result()
        assert dn == dn_e and np.array_equal(dlab, dlab_e)
