"""GPU parity of the nucleus-candidate stage (nsgb_nucleus_candidates, the tail of
HistologicalEntities::plFindNucleusCandidates, HistologicalEntities.cpp:195-275) against the
oracle's composition of the restated steps, bit-exact."""
import ctypes as C

import numpy as np
import pytest

import candidates_inputs as ci

pytestmark = pytest.mark.gpu


def to_dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def check(nsgb, oracle, rc, rc_open, rbc, *params):
    seg, n = nsgb.nucleus_candidates(to_dev(rc), to_dev(rc_open), to_dev(rbc), *params)
    exp, n_exp = oracle.nucleus_candidates(rc, rc_open, rbc, *params)
    assert n == n_exp
    assert np.array_equal(seg.cpu().numpy(), exp)
    return n, exp


@pytest.mark.parametrize("shape,n_ell", [((1024, 1024), 360), ((300, 400), 40), ((37, 61), 3), ((2048, 1536), 1100)])
def test_candidates_tiles(nsgb, oracle, shape, n_ell):
    rc, rc_open, rbc = ci.tile(shape[0], shape[1], n_ell, 2)
    n, exp = check(nsgb, oracle, rc, rc_open, rbc)
    if shape[0] >= 300:
        assert n > 0 and exp.any()


@pytest.mark.parametrize("shape", [(1, 1), (1, 300), (300, 1), (33, 65), (129, 257), (500, 700)])
def test_candidates_noise(nsgb, oracle, shape):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    rc, rc_open, rbc = ci.noise(rng, *shape)
    check(nsgb, oracle, rc, rc_open, rbc)
    check(nsgb, oracle, rc, rc_open, rbc, 40, 60, 1, 10 ** 6)


def test_candidates_parameters_and_edges(nsgb, oracle):
    rc, rc_open, rbc = ci.tile(512, 640, 120, 4)
    for params in [(80, 45, 11, 1000), (80.5, 44.9, 30, 200), (30, 90, 1, 50), (0, 0, 0, 10 ** 7)]:
        check(nsgb, oracle, rc, rc_open, rbc, *params)
    # nothing above g1: no component kept, output all 0 (the reference's NO_CANDIDATES_LEFT)
    n, exp = check(nsgb, oracle, rc, rc_open, rbc, 255, 45)
    assert n == 0 and not exp.any()
    # every pixel a red blood cell: nothing selected, the kept count unchanged
    full = np.full_like(rbc, 255)
    n_all, _ = check(nsgb, oracle, rc, rc_open, rbc)
    n_rbc, exp = check(nsgb, oracle, rc, rc_open, full)
    assert n_rbc == n_all and not exp.any()


def test_candidates_c_abi_pitched_async(nsgb, oracle):
    """Through the C ABI: pitched rows, output written over rc_open, count on the device."""
    import torch

    from nsgb import _ffi

    lib = _ffi.lib
    H, W, P = 700, 900, 913  # odd pitch: unaligned rows
    rc, rc_open, rbc = ci.tile(H, W, 250, 6)
    exp, n_exp = oracle.nucleus_candidates(rc, rc_open, rbc)

    def pitched(a):
        t = torch.zeros((H, P), dtype=torch.uint8, device="cuda")
        t[:, :W] = torch.from_numpy(a).cuda()
        return t

    t_open, t_rc, t_rbc = pitched(rc_open), pitched(rc), pitched(rbc)
    nb = lib.nsgb_workspace_size(_ffi.OP_NUCLEUS_CANDIDATES, _ffi.U8, H, W)
    ws_t = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (ws_t.data_ptr() + 255) & ~255
    n_dev = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream()
    opts = _ffi.Opts(0, 0, 0)
    st = lib.nsgb_nucleus_candidates(t_open.data_ptr(), t_rc.data_ptr(), t_rbc.data_ptr(), t_open.data_ptr(), H, W, P,
                                     80.0, 45.0, 11, 1000, None, n_dev.data_ptr(), ws, nb,
                                     C.c_void_p(s.cuda_stream), C.byref(opts))
    assert st == 0
    assert lib.nsgb_device_status(C.c_void_p(ws), C.c_void_p(s.cuda_stream)) == 0
    assert int(n_dev.item()) == n_exp
    assert np.array_equal(t_open[:, :W].cpu().numpy(), exp)
    # the padding between rows is left alone
    assert not t_open[:, W:].any()


def test_candidates_after_device_opening(nsgb, oracle):
    """S1 from rc: the device opening with the 19 x 19 disk as the marker, as the reference
    builds it (HistologicalEntities.cpp:184-199), then the candidate stage."""
    from nsgb import disk19

    rc, _, rbc = ci.tile(1024, 1280, 450, 8)
    rc_open = nsgb.morphOpen(to_dev(rc), disk19())
    exp_open = oracle.morph_open(rc, disk19())
    assert np.array_equal(rc_open.cpu().numpy(), exp_open)
    seg, n = nsgb.nucleus_candidates(to_dev(rc), rc_open, to_dev(rbc))
    exp, n_exp = oracle.nucleus_candidates(rc, exp_open, rbc)
    assert n == n_exp and n > 0
    assert np.array_equal(seg.cpu().numpy(), exp)
