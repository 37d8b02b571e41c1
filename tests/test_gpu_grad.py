"""Differentiable float32 reconstruction on the GPU: forward values and provenance, and the
adjoint, bit-exact against the oracle; the adjoint against float64 central finite
differences; the full workload (16 x 2048 x 2048) and the autograd binding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
INT_MIN = np.iinfo(np.int32).min


def _inputs(kind, shape, seed=0):
    from nsgb import synth

    if kind == "tie_free":
        mask, marker = synth.float_pair(shape, seed)
        return marker, mask
    rng = np.random.default_rng(seed)
    mask = rng.random(shape, dtype=np.float32)
    marker = (mask * rng.uniform(0.5, 1.0, shape)).astype(np.float32)
    if kind == "ties":
        mask = (np.floor(mask * 8) / 8).astype(np.float32)
        marker = (np.floor(marker * 8) / 8).astype(np.float32)
    elif kind == "negative":
        marker = (marker - 1.0).astype(np.float32)
        mask = (mask - 0.2).astype(np.float32)
    return marker, mask


@pytest.mark.parametrize("kind", ["tie_free", "ties", "negative"])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("shape", [(3, 200, 300), (1, 33, 65), (257, 129)])
def test_forward_and_adjoint_match_oracle(nsgb, oracle, kind, conn, shape):
    import torch

    marker, mask = _inputs(kind, shape, 2)
    out, prov = nsgb.recon_f32(torch.from_numpy(marker).cuda(), torch.from_numpy(mask).cuda(), conn)
    R, P = oracle.recon_f32_prov(marker, mask, conn)
    assert np.array_equal(out.cpu().numpy(), R)
    assert np.array_equal(prov.cpu().numpy(), P)
    g = np.random.default_rng(3).standard_normal(shape).astype(np.float32)
    dm, dk = nsgb.recon_f32_backward(torch.from_numpy(g).cuda(), prov)
    em, ek = oracle.recon_f32_grad(g, P)
    assert np.array_equal(dm.cpu().numpy(), em)
    assert np.array_equal(dk.cpu().numpy(), ek)


@pytest.mark.parametrize("conn", [4, 8])
def test_adjoint_matches_finite_differences(nsgb, oracle, conn):
    """512 random pixels, central differences with h = 1e-4 evaluated in float64 on the CPU;
    pixels whose provenance changes at x +- h are rejected (counted)."""
    import torch

    marker, mask = _inputs("tie_free", (512, 512), 7)
    out, prov = nsgb.recon_f32(torch.from_numpy(marker).cuda(), torch.from_numpy(mask).cuda(), conn)
    g = np.random.default_rng(8).standard_normal(mask.shape).astype(np.float32)
    dm, dk = nsgb.recon_f32_backward(torch.from_numpy(g).cuda(), prov)
    dm, dk = dm.cpu().numpy().ravel(), dk.cpu().numpy().ravel()
    idx = np.random.default_rng(9).choice(mask.size, 512, replace=False)
    fm, fk, vm, vk = oracle.recon_fd(marker, mask, g, conn, idx, h=1e-4)
    rejected = int((~vm).sum() + (~vk).sum())
    print(f"finite differences: {rejected} of 1024 rejected (provenance changes within h)")
    assert rejected < 40
    # the adjoint is the exact sum of each source's contributions rounded once to float32, so it
    # lies within half a float32 ulp of the float64 central differences (whose own error is
    # below 1e-10 here) at every pixel whose provenance does not change within +-h
    for fd, d, v in ((fm, dm[idx], vm), (fk, dk[idx], vk)):
        half_ulp = (np.nextafter(np.abs(d), np.float32(np.inf)) - np.abs(d)).astype(np.float64) / 2
        assert np.all((np.abs(fd - d) <= half_ulp + 1e-10)[v])
    assert np.count_nonzero(dm[idx][vm]) + np.count_nonzero(dk[idx][vk]) > 100


def test_full_workload_16x2048(nsgb, oracle):
    """16 images of 2048 x 2048, mask uniform in [0,1), marker = mask * U[0.5,1), g ~ N(0,1):
    values, provenance and both gradients bit-exact against the oracle; the backward costs at
    most twice the forward."""
    import torch

    from nsgb import synth

    mask, marker = synth.float_pair((16, 2048, 2048), 0)
    g = np.random.default_rng(0).standard_normal(mask.shape).astype(np.float32)
    mk, ms, gg = (torch.from_numpy(a).cuda() for a in (marker, mask, g))
    nsgb.recon_f32(mk, ms, 8)  # warm-up
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    e[0].record()
    out, prov = nsgb.recon_f32(mk, ms, 8)
    e[1].record()
    dm, dk = nsgb.recon_f32_backward(gg, prov)
    e[2].record()
    torch.cuda.synchronize()
    t_fwd, t_bwd = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    print(f"forward {t_fwd:.2f} ms, backward {t_bwd:.2f} ms")
    R, P = oracle.recon_f32_prov(marker, mask, 8)
    assert np.array_equal(out.cpu().numpy(), R)
    assert np.array_equal(prov.cpu().numpy(), P)
    em, ek = oracle.recon_f32_grad(g, P)
    assert np.array_equal(dm.cpu().numpy(), em)
    assert np.array_equal(dk.cpu().numpy(), ek)
    assert t_bwd <= 2.0 * t_fwd


def test_autograd_binding(nsgb):
    import torch

    from nsgb.autograd import imreconstruct_f32

    marker, mask = _inputs("tie_free", (2, 96, 128), 4)
    mk = torch.from_numpy(marker).cuda().requires_grad_()
    ms = torch.from_numpy(mask).cuda().requires_grad_()
    out = imreconstruct_f32(mk, ms, 8)
    g = torch.randn_like(out)
    (out * g).sum().backward()
    _, prov = nsgb.recon_f32(mk.detach(), ms.detach(), 8)
    dm, dk = nsgb.recon_f32_backward(g, prov)
    assert torch.equal(mk.grad, dm) and torch.equal(ms.grad, dk)
    # every output value is copied from exactly one input: gradients conserve the total
    assert abs(float(mk.grad.sum() + ms.grad.sum()) - float(g.sum())) < 1e-2


def test_adjoint_sum_is_exact(nsgb, oracle):
    """Sums that a coarse fixed point would get wrong: cancellation that leaves a 2^-70 term, a
    tie between two floats (ties to even), and contributions in scattered order; the GPU matches
    the oracle's exact sums bit for bit."""
    import torch

    g = np.zeros((4, 8), np.float32)
    g[0, :4] = [2.0**30, -(2.0**30), 2.0**-70, 3.0 * 2.0**-60]
    g[1, :3] = [1.0, 2.0**-24, 0.0]
    g[2] = np.random.default_rng(3).standard_normal(8).astype(np.float32)
    g[3] = -g[2][::-1]
    prov = np.zeros((4, 8), np.int32)
    prov[0, :4] = 3
    prov[0, 4:] = ~np.arange(4, 8)
    prov[1, :] = ~9
    prov[2:, :] = 17  # g[3] cancels g[2] exactly
    dm, dk = nsgb.recon_f32_backward(torch.from_numpy(g).cuda(), torch.from_numpy(prov).cuda())
    em, ek = oracle.recon_f32_grad(g, prov)
    assert dm.cpu().numpy().tobytes() == em.tobytes() and dk.cpu().numpy().tobytes() == ek.tobytes()
    assert em.ravel()[3] == np.float32(2.0**-70 + 3.0 * 2.0**-60)
    assert ek.ravel()[9] == np.float32(1.0) and em.ravel()[17] == 0.0


def test_adjoint_rejects_huge_gradients(nsgb):
    import torch

    g = torch.full((8, 8), 2.0**31, device="cuda")
    prov = torch.zeros((8, 8), dtype=torch.int32, device="cuda")
    with pytest.raises(nsgb.NsgbError):
        nsgb.recon_f32_backward(g, prov)


def test_bad_provenance_is_reported(nsgb):
    import torch

    g = torch.ones((8, 8), device="cuda")
    prov = torch.full((8, 8), 64, dtype=torch.int32, device="cuda")  # out of range
    with pytest.raises(nsgb.NsgbError):
        nsgb.recon_f32_backward(g, prov)
