"""The bounded waits of the inverse z pass, made to run out on purpose.

k_c2r_zp stages each step's lines with a bulk copy that completes on an
mbarrier and waits for it a bounded number of polls.  The test hook
prc_d2z_test_withhold_copy makes one CTA skip its first copy, so its wait
runs out for real with nothing in flight (no fault, no hang: the wait gives
up, the CTA sets the error word and returns).  The call must report it, and
the context must stay usable.
"""
import numpy as np
import pytest

import prc_d2z
from prc_d2z import _lib, fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [32, 64, 128])
def test_forward_reports_a_wait_that_ran_out(N):
    import torch
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=10, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
    delta = torch.from_numpy(fields.gaussian_field(N, box, seed=31)).cuda()
    L = _lib.load()
    with prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=4) as ctx:
        z_ref, am_ref, _ = ctx.forward(delta)
        z_ref, am_ref = z_ref.cpu().numpy(), am_ref.cpu().numpy()
        _lib.check(L.prc_d2z_test_withhold_copy(1))
        try:
            with pytest.raises(prc_d2z.PrcError) as ei:
                ctx.forward(delta)
        finally:
            L.prc_d2z_test_withhold_copy(0)
        assert ei.value.code == _lib.PRC_ERR_CUDA
        assert "wait limit" in str(ei.value)
        # the context is usable and the error word was cleared
        z, am, _ = ctx.forward(delta)
        torch.cuda.synchronize()
        assert np.array_equal(z.cpu().numpy(), z_ref)
        assert np.array_equal(am.cpu().numpy(), am_ref)


def test_withhold_hook_rejects_negative():
    L = _lib.load()
    assert L.prc_d2z_test_withhold_copy(-1) == _lib.PRC_ERR_INVALID
    assert L.prc_d2z_test_withhold_copy(0) == _lib.PRC_OK
