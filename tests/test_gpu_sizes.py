"""The grid sizes three times a power of two above 192: 384^3 (450 Mpc/h) and
768^3 (900 Mpc/h), 32 radii from 2 cells to 60 Mpc/h at the 512^3 workload's
cell size (1.17 Mpc/h), against the FP64 restatement of the chain (cuFFT in
double precision; test-only).  Their column transforms are mixed radix with a
radix-3 stage (384: 4 4 4 3 2 on 32 lanes x 16 columns; 768: 4 4 4 4 3 on
64 lanes x 8 columns) and their z lines use the paired C2R of lengths 192 and
384, so every pass runs a plan that no other grid size runs.

Forward: delta_R within 1e-5 relative RMS of FP64 for the first, a middle and
the last radius; zreion within eps_z = A 1e-5 max|delta_R| + 2 ulp and the same
argmax on every cell whose FP64 top-two margin exceeds eps_z; x_i(z) within
1e-4; for the default radius batch and for 32 radii in one sweep.
Adjoint: dL/d delta_lin within 1e-5 relative L2 of the FP64 adjoint."""
import math

import numpy as np
import pytest

import prc_d2z
from fp64_chain import chain as _fp64_chain
from fp64_chain import kmag, tophat64
from prc_d2z import fields

pytestmark = pytest.mark.gpu
H_ = 0.68
ZETA = 80.5404
NR = 32


def _setup(N, box):
    p = prc_d2z.Parameters(N=N, Nscales=NR, BoxSize=box, Rmin=2.0)
    cl = prc_d2z.CLParameters(Rmax=60.0, zeta=ZETA, M_min=1e9 / H_)
    return p, cl, float(np.float32(box) / np.float32(H_))


@pytest.mark.parametrize("N,box,need_gb", [(384, 450.0, 24), (768, 900.0, 110)])
def test_forward_against_fp64(N, box, need_gb):
    import torch
    free, _ = torch.cuda.mem_get_info()
    if free < need_gb * 2 ** 30:
        pytest.skip("not enough device memory for the FP64 restatement")
    assert N in prc_d2z.supported_sizes()
    p, cl, box_mpc = _setup(N, box)
    delta = fields.gaussian_field(N, box, seed=1, backend="torch").contiguous()
    check = (0, NR // 2, NR - 1)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        t = ctx.tables
        z, am, _ = ctx.forward(delta)
        dRs = {r: ctx.smooth(delta, r) for r in check}
        torch.cuda.synchronize()
        zo, amo, gap, dmax, keep = _fp64_chain(delta, box_mpc, t.radii_mpc, t.barrier_a, t.barrier_b, t.DInit,
                                               check)
        for r in check:
            d = dRs[r].double() - keep[r]
            rel = math.sqrt(float((d * d).mean()) / float((keep[r] * keep[r]).mean()))
            assert rel < 1e-5, (r, rel)
        del keep, dRs
        eps = t.barrier_a * 1e-5 * dmax + 2 * torch.abs(zo).float().nextafter(
            torch.tensor(math.inf, device=zo.device)).sub(torch.abs(zo).float()).double()
        clear = gap > eps
        frac_near = 1.0 - float(clear.double().mean())
        assert frac_near < 0.05, frac_near
        assert float((zo > 0).double().mean()) > 0.1
        _, x_64, _ = ctx.history(zo.float().contiguous())
        for B in (0, NR):
            if B:
                ctx.tune(B, 0)
                z, am, _ = ctx.forward(delta)
            dz = (z.double() - zo).abs()
            assert bool((dz[clear] <= eps[clear]).all()), (B, float(dz[clear].max()))
            assert bool((am[clear] == amo[clear]).all()), B
            _, x_gpu, _ = ctx.history(z)
            dx = float(np.max(np.abs(x_gpu.astype(np.float64) - x_64.astype(np.float64))))
            assert dx <= 1e-4, (B, dx)
            print(f"N={N}, radius batch {B or 'default'}: near-barrier fraction {frac_near:.2e}, "
                  f"max |dz| on clear cells {float(dz[clear].max()):.3e}, max |dx_i| {dx:.2e}")


def test_adjoint_against_fp64_384():
    """dL/d delta_lin at 384^3 x 32 radii, L = mean((z - z_t)^2), against
    (1/D) sum_r IDFT(W_r DFT(A g [argmax == r])) in FP64."""
    import torch
    N, box = 384, 450.0
    free, _ = torch.cuda.mem_get_info()
    if free < 24 * 2 ** 30:
        pytest.skip("not enough device memory for the FP64 adjoint")
    p, cl, box_mpc = _setup(N, box)
    delta = fields.gaussian_field(N, box, seed=1, backend="torch").contiguous()
    target = fields.gaussian_field(N, box, seed=2, backend="torch").contiguous()
    with prc_d2z.Delta2Zreion.from_parameters(p, cl, argmax=True) as ctx:
        t = ctx.tables
        z, am, _ = ctx.forward(delta)
        g = (2.0 * (z.double() - target.double()) / N ** 3).float().contiguous()
        grad, dB = ctx.backward(g, am)
        torch.cuda.synchronize()
    km = kmag(N, box_mpc, delta.device)
    g64 = g.double()
    acc = torch.zeros((N, N, N // 2 + 1), dtype=torch.complex128, device=delta.device)
    dB64 = np.zeros(NR)
    for r in range(NR):
        m = am == r
        if bool(m.any()):
            W = tophat64(km * t.radii_mpc[r])
            W[0, 0, 0] = 0.0
            gr = torch.where(m, t.barrier_a * g64, torch.zeros_like(g64))
            dB64[r] = float(gr.sum())
            acc += W * torch.fft.rfftn(gr)
            del W, gr
    ref = torch.fft.irfftn(acc, s=(N, N, N)) / t.DInit
    del acc
    rel = float(torch.linalg.vector_norm(grad.double() - ref) / torch.linalg.vector_norm(ref))
    assert rel < 1e-5, rel
    np.testing.assert_allclose(dB, dB64, rtol=1e-5, atol=1e-9 * np.abs(dB64).max())
    print(f"N={N}: FP64-adjoint relative error {rel:.2e}")
