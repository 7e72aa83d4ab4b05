"""The device's pow of the material laws equals the host build of the same correctly
rounded pow (dumux_gb300/csrc/crpow.cuh) bit for bit."""
import numpy as np
import pytest

import oracle
from dumux_gb300 import device_pow

pytestmark = pytest.mark.gpu


def test_device_pow_equals_host_correctly_rounded_pow():
    rng = np.random.default_rng(7)
    n = 400000
    x = np.concatenate([rng.uniform(0, 1, n), np.exp(rng.uniform(-40, 40, n)),
                        rng.integers(1, 2 ** 20, n // 4).astype(np.float64)])
    y = np.concatenate([rng.choice([-0.5, 4.0, 2.0, 3.0, -1.5, 1.0 / 2.7, 2.7, 0.63, 1.59], n),
                        rng.uniform(-15, 15, n), rng.choice([2.0, 3.0, 1.5, -3.0], n // 4)])
    sv = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 2.0, -2.0, 0.5, -0.5, 3.0, 1e-310, 5e-324, 1.7e308])
    xs, ys = (a.ravel() for a in np.meshgrid(sv, sv))
    x = np.concatenate([x, xs])
    y = np.concatenate([y, ys])
    d = device_pow(x, y)
    h = oracle.pow_batch(x, y, oracle.POW_CORRECTLY_ROUNDED)
    same = (d.view(np.int64) == h.view(np.int64)) | (np.isnan(d) & np.isnan(h))
    assert same.all(), np.nonzero(~same)[0][:10]
