"""The large single-image workload: 16384 x 16384 (268 Mpixel) with about 102k ellipses,
hole filling by reconstruction by erosion (marker = image on the border, max elsewhere) in
4- and 8-connectivity, threshold > 128 (scaled with the dtype) and bwlabel (8-connected,
raster relabel) of the result, all device-resident; plus bwlabel of the dark objects
(image <= 128: about 69k components, the 102k ellipses
minus the overlapping ones).  Every stage bit-exact against the oracle."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 16384


@pytest.fixture(scope="module")
def image_u8():
    from nsgb import synth

    mask, _ = synth.tile_u8(N, N, int(round(N * N / 2621)), 0)
    return mask


def _oracle_stage(oracle, img, conn, thr):
    fill = oracle.imfill_holes(img, False, conn)
    b = oracle.threshold_gt(fill, thr)
    lab, n = oracle.bwlabel2(b, 8, True)
    return fill, lab, n


@pytest.mark.parametrize("dtype", ["u8", "u16", "i32"])
def test_large_fill_threshold_label(nsgb, oracle, image_u8, dtype):
    import torch

    from nsgb import synth

    scale = {"u8": 1, "u16": 257, "i32": 1000}[dtype]
    img = image_u8 if dtype == "u8" else synth.scale(image_u8, dtype)[0]
    thr = 128.0 * scale
    with ThreadPoolExecutor(3) as ex:
        futs = {conn: ex.submit(_oracle_stage, oracle, img, conn, thr) for conn in (4, 8)}
        dark = ex.submit(lambda: oracle.bwlabel2(255 - oracle.threshold_gt(img, thr), 8, True))
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
        for conn in (4, 8):
            fill_e, lab_e, n_e = futs[conn].result()
            fill_g, lab_g, n_g = got[conn]
            assert np.array_equal(fill_g, fill_e), f"fill conn={conn}"
            assert n_g == n_e and np.array_equal(lab_g, lab_e), f"labels conn={conn}"
        dlab_e, dn_e = dark.result()
        assert dn == dn_e and np.array_equal(dlab, dlab_e)
        assert dn > 50000
