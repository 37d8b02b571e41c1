"""GPU against the reference's own code: the outputs that the reference's nscale::imreconstruct,
imreconstructBinary, imfillHoles, imhmin, bwselect, bwlabel2 and bwareaopen2 produced
(compiled unmodified from its sources, oracle/build_ref.sh) are committed as fixtures:

* tests/golden/ref_recon_cases.npz: 308 small cases, every dtype, 4 / 8-connected, compared
  bit for bit (float zeros by sign too);
* tests/golden/ref_recon_digests.json: SHA-256 digests of the reference's outputs on the
  workloads (c0 reconstruction, the c1 chain stages and the inverted chain, every c2 tile's
  chain in u8 / u16 / i32, the c3 f32 reconstruction per image).  The c4 digests are checked
  in tests/test_gpu_large.py.
The i32 hole-fill cases are compared under the saturating CV_32S reading (OpenCV's own
wrap-around makes the reference's imfillHoles<int> return INT_MIN everywhere; the oracle
tests pin both readings).
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")


def to_dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def same(got, exp):
    got = got.cpu().numpy() if hasattr(got, "cpu") else np.asarray(got)
    return got.dtype == exp.dtype and got.shape == exp.shape and got.tobytes() == exp.tobytes()


@pytest.fixture(scope="module")
def digests():
    return json.load(open(os.path.join(GOLDEN, "ref_recon_digests.json")))


def test_cases_match_reference(nsgb):
    d = np.load(os.path.join(GOLDEN, "ref_recon_cases.npz"))
    meta = json.loads(str(d["meta"]))
    bad = []
    for k, c in enumerate(meta):
        if c.get("reading") == "wrap":
            continue
        ins = [to_dev(d[name]) for name in c["inputs"]]
        op, conn = c["op"], c["conn"]
        if op == "imreconstruct":
            got = nsgb.imreconstruct(ins[0], ins[1], conn)
        elif op == "imreconstructBinary":
            got = nsgb.imreconstructBinary(ins[0], ins[1], conn)
        elif op == "imfillHoles":
            got = nsgb.imfillHoles(ins[0], c["binary"], conn)
        elif op == "imhmin":
            got = nsgb.imhmin(ins[0], c["h"], conn)
        else:
            got = nsgb.bwselect(ins[0], ins[1], conn)
        if not same(got, d[f"out{k}"]):
            bad.append(c)
    assert not bad, bad[:5]


def test_c0_c1_match_reference_digests(nsgb, digests):
    import workloads as W

    marker, mask = W.c0()
    for conn in (4, 8):
        got = nsgb.imreconstruct(to_dev(marker), to_dev(mask), conn).cpu().numpy()
        assert W.digest(got) == digests["c0"][f"recon{conn}"], conn
    runs = {"c1_1024": W.c1(1024, 400, 0), "c1_2048_s4": W.c1(2048, 1500, 4), "c1_4096": W.c1()}
    for name, (mk, ms) in runs.items():
        assert W.chain_digest(nsgb.chain(to_dev(mk), to_dev(ms))) == digests["c1"][name], name
        imk, ims = W.inverted(ms)
        assert W.chain_digest(nsgb.chain(to_dev(imk), to_dev(ims))) == digests["c1"][name + "_inverted"], name


@pytest.mark.parametrize("dtype", ["u8", "u16", "i32"])
def test_c2_batch_matches_reference_digests(nsgb, digests, dtype):
    """Every tile of the 256-tile batch, through the batched chain, against the reference."""
    from concurrent.futures import ThreadPoolExecutor

    import workloads as W

    sizes = W.c2_sizes()
    with ThreadPoolExecutor() as ex:
        tiles = list(ex.map(lambda i: W.c2_tile(i, dtype, sizes), range(256)))
    res = nsgb.chain_batch([to_dev(k) for k, _ in tiles], [to_dev(m) for _, m in tiles], thr=128.0 * W.SCALE[dtype])
    got = [W.chain_digest(r) for r in res]
    bad = [i for i in range(256) if got[i] != digests["c2"][dtype][i]]
    assert not bad, bad[:10]


def test_c3_forward_matches_reference_digests(nsgb, digests):
    import workloads as W

    marker, mask = W.c3()
    out, _ = nsgb.recon_f32(to_dev(marker), to_dev(mask), 8)
    out = out.cpu().numpy()
    got = [W.digest(out[b]) for b in range(out.shape[0])]
    assert got == digests["c3"]["recon8"]
