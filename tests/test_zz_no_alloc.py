"""prc_d2z_forward_static: the forward path that allocates no device memory.

It serves callers that cannot allocate device memory when they need the
result (a host framework that owns all device memory, or a stage that cannot
pay for cudaMalloc/cudaFree).  Called through the C ABI with device pointers,
twice in a row on different fields, its zreion and argmax must equal those of
prc_d2z_forward (exactly: both run the same kernels on the same data, and the
grouping of radii into sweeps does not change any result).  This file is
collected last so that a failing run stops after every other test.
"""
import ctypes

import numpy as np
import pytest

import prc_d2z
from prc_d2z import _lib, fields

pytestmark = pytest.mark.gpu


def _static_forward(N, t, box_mpc, delta_dev, z_dev, am_dev):
    L = _lib.load()
    R = np.ascontiguousarray(t.radii_mpc, np.float64)
    B = np.ascontiguousarray(t.barrier_b, np.float64)
    return L.prc_d2z_forward_static(N, len(R), box_mpc, R.ctypes.data, B.ctypes.data, t.barrier_a, t.DInit,
                                    ctypes.c_void_p(delta_dev.data_ptr()), ctypes.c_void_p(z_dev.data_ptr()),
                                    ctypes.c_void_p(am_dev.data_ptr()) if am_dev is not None else None, None)


def _case(N):
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=12, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
    return p, cl, prc_d2z.compute_tables(p, cl), float(np.float32(box) / np.float32(0.68))


# 32 and 64 run the bulk-copy-staged inverse z pass, 12 and 24 the
# shared-memory-staged one
@pytest.mark.parametrize("N", [12, 24, 32, 64])
def test_static_workspace_forward_matches_forward_twice(N):
    import torch
    p, cl, t, box_mpc = _case(N)
    for seed in (21, 22):  # two calls in a row, different inputs
        delta = fields.gaussian_field(N, p.BoxSize, seed=seed)
        with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
            z_ref, am_ref, _ = ctx.forward(delta)
        d = torch.from_numpy(delta).cuda()
        z = torch.full(d.shape, -7.0, dtype=torch.float32, device="cuda")
        am = torch.full(d.shape, 77, dtype=torch.uint8, device="cuda")
        _lib.check(_static_forward(N, t, box_mpc, d, z, am))
        torch.cuda.synchronize()
        assert np.array_equal(z.cpu().numpy(), z_ref)
        assert np.array_equal(am.cpu().numpy(), am_ref)


@pytest.mark.parametrize("N", [24, 64])
def test_static_workspace_forward_without_argmax(N):
    """argmax is optional: zreion alone still equals prc_d2z_forward's."""
    import torch
    p, cl, t, box_mpc = _case(N)
    delta = fields.gaussian_field(N, p.BoxSize, seed=23)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        z_ref, _, _ = ctx.forward(delta)
    d = torch.from_numpy(delta).cuda()
    z = torch.full(d.shape, -7.0, dtype=torch.float32, device="cuda")
    _lib.check(_static_forward(N, t, box_mpc, d, z, None))
    torch.cuda.synchronize()
    assert np.array_equal(z.cpu().numpy(), z_ref)


def test_static_workspace_reports_a_wait_that_ran_out():
    """A z-pass CTA whose staging copy never comes (withheld by the test hook,
    so nothing is in flight) gives up after its bounded wait; the call reports
    PRC_ERR_CUDA through the static error word, and the next call is exact."""
    import torch
    N = 32
    p, cl, t, box_mpc = _case(N)
    L = _lib.load()
    delta = fields.gaussian_field(N, p.BoxSize, seed=24)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        z_ref, am_ref, _ = ctx.forward(delta)
    d = torch.from_numpy(delta).cuda()
    z = torch.zeros(d.shape, dtype=torch.float32, device="cuda")
    am = torch.zeros(d.shape, dtype=torch.uint8, device="cuda")
    _lib.check(L.prc_d2z_test_withhold_copy(1))
    try:
        st = _static_forward(N, t, box_mpc, d, z, am)
    finally:
        L.prc_d2z_test_withhold_copy(0)
    assert st == _lib.PRC_ERR_CUDA
    assert b"wait limit" in L.prc_last_error()
    _lib.check(_static_forward(N, t, box_mpc, d, z, am))
    torch.cuda.synchronize()
    assert np.array_equal(z.cpu().numpy(), z_ref)
    assert np.array_equal(am.cpu().numpy(), am_ref)


def test_static_workspace_rejects_large_grids():
    import torch
    L = _lib.load()
    R = np.array([2.0, 3.0])
    B = np.array([5.0, 6.0])
    buf = torch.zeros(8, device="cuda")
    st = L.prc_d2z_forward_static(128, 2, 100.0, R.ctypes.data, B.ctypes.data, 0.75, 1.0,
                                  ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()), None, None)
    assert st == _lib.PRC_ERR_INVALID
    assert b"N=64" in L.prc_last_error()
