"""GPU disorder generation (make_corr_rand_3d with the transforms on the device) against the host
form and the Ooura-FFT golden vectors of the reference's own filter."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "corr3d_golden.npz")


@pytest.mark.parametrize("n1,n2,n3,xi,uniform", [(8, 8, 4, 3.0, True), (10, 10, 6, 3.0, True),
                                                 (24, 24, 24, 3.0, True), (32, 32, 32, 2.0, False),
                                                 (96, 96, 8, 3.0, True), (12, 12, 12, 0.0, True)])
def test_gpu_generator_equals_host(engine_mod, n1, n2, n3, xi, uniform):
    jc = engine_mod
    for seed in (1, 17):
        host = jc.corr_rand_3d(n1, n2, n3, xi, seed, uniform, 2.0)
        dev = jc.corr_rand_3d(n1, n2, n3, xi, seed, uniform, 2.0, gpu=True)
        assert np.abs(dev - host).max() < 1e-12


def _golden_cases():
    g = np.load(GOLDEN)
    cases = {}
    for k in g.files:
        name, part = k.split("__")
        cases.setdefault(name, {})[part] = g[k]
    for name, d in cases.items():
        dims, xi, s, u, m = name.split("_")
        n1, n2, n3 = (int(v) for v in dims[1:].split("x"))
        yield (n1, n2, n3, float(xi[2:]), int(s[1:]), bool(int(u[1:])), float(m[1:])), d


def test_gpu_generator_matches_golden(engine_mod):
    """Against the reference's filter compiled around its vendored Ooura FFT (committed vectors)."""
    jc = engine_mod
    n = 0
    for (n1, n2, n3, xi, seed, uni, mx), d in _golden_cases():
        x = jc.corr_rand_3d(n1, n2, n3, xi, seed, uni, mx, gpu=True).reshape(-1)
        stride = int(d["stride"][0])
        np.testing.assert_allclose(x[::stride], d["values"], rtol=0, atol=1e-12)
        np.testing.assert_allclose([x.sum(), (x * x).sum()], d["sum"], rtol=1e-12, atol=1e-9)
        n += 1
    assert n >= 5


def test_gpu_generator_rejects_bad_extents(engine_mod):
    jc = engine_mod
    with pytest.raises(jc.J1J2CError):
        jc.corr_rand_3d(0, 4, 4, 3.0, 1, gpu=True)
