"""Batched form: many uneven tiles in one reconstruction launch and one launch per labelling
stage must give, tile by tile, exactly the single-tile results (checked against the oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tiles(dtype, sizes, seed0=0):
    from nsgb import synth

    out = []
    for k, (h, w) in enumerate(sizes):
        m8, k8 = synth.tile_u8(h, w, synth.ellipses_for(h, w), seed0 + k)
        if dtype == "u8":
            out.append((m8, k8))
        else:
            out.append(synth.scale(m8, dtype))
    return out


SIZES = [(256, 300), (33, 65), (1, 97), (97, 1), (300, 256), (512, 777), (64, 64), (129, 31), (700, 403), (2, 2)]


@pytest.mark.parametrize("dtype", ["u8", "u16", "i32"])
def test_chain_batch_matches_single_tiles(nsgb, oracle, dtype):
    import torch

    tiles = _tiles(dtype, SIZES)
    scale = {"u8": 1, "u16": 257, "i32": 1000}[dtype]
    res = nsgb.chain_batch([torch.from_numpy(k).cuda() for _, k in tiles],
                           [torch.from_numpy(m).cuda() for m, _ in tiles], thr=128 * scale)
    for (m, k), got in zip(tiles, res):
        exp = oracle.chain(k, m, thr=128 * scale)
        assert np.array_equal(got["recon"].cpu().numpy(), exp["recon"])
        assert np.array_equal(got["fill"].cpu().numpy(), exp["fill"])
        assert np.array_equal(got["labels"].cpu().numpy(), exp["labels"])
        assert np.array_equal(got["area"].cpu().numpy(), exp["area"])
        assert got["n_labels"] == exp["n_labels"] and got["n_kept"] == exp["n_kept"]


@pytest.mark.parametrize("fill_conn", [4, 8])
def test_chain_batch_hole_fill_edges(nsgb, oracle, fill_conn):
    """The batch's bit-plane hole fill (a flood from outside each image): widths around the
    32-pixel words and the 1024-pixel flood tiles, one-pixel images, heights around the 32-row
    tiles, inverted tiles (the open class is the whole background, so the flood crosses every
    image) and both fill connectivities, against the oracle tile by tile."""
    import torch

    sizes = [(31, 1023), (32, 1024), (33, 1025), (65, 2049), (1, 1), (1, 40), (40, 1), (100, 31), (100, 33),
             (64, 3000), (95, 64), (257, 1100)]
    tiles = _tiles("u8", sizes, 70)
    # every other tile inverted: dark background, bright objects
    tiles = [((255 - m).astype(np.uint8), np.maximum((255 - m).astype(np.int16) - 10, 0).astype(np.uint8))
             if i % 2 else (m, k) for i, (m, k) in enumerate(tiles)]
    res = nsgb.chain_batch([torch.from_numpy(k).cuda() for _, k in tiles],
                           [torch.from_numpy(m).cuda() for m, _ in tiles], fill_conn=fill_conn)
    for i, ((m, k), got) in enumerate(zip(tiles, res)):
        exp = oracle.chain(k, m, fill_conn=fill_conn)
        assert np.array_equal(got["fill"].cpu().numpy(), exp["fill"]), (i, sizes[i])
        assert np.array_equal(got["labels"].cpu().numpy(), exp["labels"]), (i, sizes[i])
        assert got["n_labels"] == exp["n_labels"] and got["n_kept"] == exp["n_kept"]


@pytest.mark.parametrize("conn", [4, 8])
def test_reconstruct_batch_matches_oracle(nsgb, oracle, conn):
    import torch

    tiles = _tiles("u8", SIZES, 50)
    outs = nsgb.imreconstructQueueThroughput([torch.from_numpy(k).cuda() for _, k in tiles],
                                             [torch.from_numpy(m).cuda() for m, _ in tiles], conn)
    for (m, k), got in zip(tiles, outs):
        assert np.array_equal(got.cpu().numpy(), oracle.imreconstruct(k, m, conn))


def test_batch_of_one_and_replay(nsgb, oracle):
    import torch

    (m, k), = _tiles("u8", [(300, 500)], 7)
    recon = torch.from_numpy(k).cuda()
    plan = nsgb.BatchPlan([recon], [torch.from_numpy(m).cuda()])
    exp = oracle.chain(k, m)
    for _ in range(2):  # the prepared plan is replayed; the marker is restored in between
        recon.copy_(torch.from_numpy(k).cuda())
        nl, nk = plan.chain()
        assert nl[0] == exp["n_labels"] and nk[0] == exp["n_kept"]
        assert np.array_equal(plan.labels[0].cpu().numpy(), exp["labels"])
        assert np.array_equal(recon.cpu().numpy(), exp["recon"])


@pytest.mark.parametrize("dtype", ["u8", "u16", "i32"])
def test_chain_batch_full_workload(nsgb, oracle, dtype):
    """The full batched workload: 256 tiles with H, W i.i.d. uniform in [256, 4096] (tile i
    from seed i, one ellipse per 2800 px^2), every tile checked against the oracle."""
    import torch
    from concurrent.futures import ThreadPoolExecutor

    from nsgb import synth

    h, w = synth.tile_sizes(256, 256, 4096, 0xC2)
    scale = {"u8": 1, "u16": 257, "i32": 1000}[dtype]

    def make(i):
        m, k = synth.tile_u8(int(h[i]), int(w[i]), synth.ellipses_for(int(h[i]), int(w[i])), i)
        return (m, k) if dtype == "u8" else synth.scale(m, dtype)

    with ThreadPoolExecutor() as ex:
        tiles = list(ex.map(make, range(256)))
    res = nsgb.chain_batch([torch.from_numpy(k).cuda() for _, k in tiles],
                           [torch.from_numpy(m).cuda() for m, _ in tiles], thr=128 * scale)

    def check(i):
        m, k = tiles[i]
        exp = oracle.chain(k, m, thr=128 * scale)
        got = res[i]
        return (np.array_equal(got["recon"].cpu().numpy(), exp["recon"])
                and np.array_equal(got["fill"].cpu().numpy(), exp["fill"])
                and np.array_equal(got["labels"].cpu().numpy(), exp["labels"])
                and np.array_equal(got["area"].cpu().numpy(), exp["area"])
                and got["n_labels"] == exp["n_labels"] and got["n_kept"] == exp["n_kept"])

    torch.cuda.synchronize()
    with ThreadPoolExecutor() as ex:
        ok = list(ex.map(check, range(256)))
    assert all(ok), [i for i, v in enumerate(ok) if not v][:10]
