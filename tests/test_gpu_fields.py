"""The native field generator (prc_white_noise, prc_d2z_gaussian_field)
against the numpy definition in prc_d2z.fields."""
import numpy as np
import pytest

import prc_d2z
from prc_d2z import fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,seed", [(16, 1), (32, 7), (64, 123456789)])
def test_white_noise_kernel_matches_numpy(N, seed):
    w = fields.white_noise_native(N, seed).cpu().numpy()
    ref = fields.white_noise(N, seed).astype(np.float32)
    # FP64 Box-Muller on both sides; the libm and CUDA results may differ in
    # the last double bit, which survives the float32 rounding at most as 1 ulp
    ulp = np.spacing(np.abs(ref))
    assert np.all(np.abs(w - ref) <= ulp), float(np.max(np.abs(w - ref) / ulp))


@pytest.mark.parametrize("N", [32, 64, 128])
def test_native_field_matches_numpy(N):
    box = 1.5 * N
    d = fields.gaussian_field(N, box, seed=3, backend="native").cpu().numpy()
    ref = fields.gaussian_field(N, box, seed=3)
    rel = np.linalg.norm(d - ref) / np.linalg.norm(ref)
    assert rel < 2e-6, rel


def test_native_field_host_output_and_engine_reuse():
    N, box = 32, 48.0
    with prc_d2z.Delta2Zreion(N, box / 0.68, [1.0, 2.0], [0.0, 0.0], 1.0, 1.0) as eng:
        tab = fields.amplitude_table(N, box)
        a = eng.gaussian_field(5, tab)
        b = fields.gaussian_field(N, box, seed=5, backend="native", engine=eng).cpu().numpy()
        assert np.array_equal(a, b)
        with pytest.raises(prc_d2z.PrcError):
            eng.gaussian_field(5, tab[:-1])
