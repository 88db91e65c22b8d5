"""CPU tests of libj1j2cuda: the C ABI loads and exports every declared entry point, and the
host-side model helpers agree with the oracle / golden vectors (no GPU compute is called)."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "j1j2c.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(j1j2c_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine_mod):
    import ctypes
    lib = ctypes.CDLL(engine_mod.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(engine_mod.EXPORTS) | (set(syms) - set(engine_mod.EXPORTS))
    assert set(engine_mod.EXPORTS) <= set(syms)
    assert b"sm_103a" in engine_mod.lib().j1j2c_version()



def test_header_constants_match_python_mirror(engine_mod):
    """Every J1J2C_FLAG_ / START_ / AXIS_ / precision constant of the header has the same value in
    the ctypes host mirror (a flag added on one side only would silently pin the wrong path)."""
    text = open(HEADER).read()
    defs = dict(re.findall(r"#define J1J2C_((?:FLAG|START|AXIS|FP64|FP32)_[A-Z0-9_]+)\s+(-?\d+)u?",
                           text))
    assert len(defs) >= 15
    for name, value in defs.items():
        assert getattr(engine_mod, name) == int(value), name


def test_corr_rand_3d_matches_ooura_golden(engine_mod):
    g = np.load(os.path.join(ROOT, "tests", "golden", "corr3d_golden.npz"))
    n = 0
    for k in g.files:
        if not k.endswith("__values"):
            continue
        name = k[:-len("__values")]
        dims, xi, s, u, m = name.split("_")
        n1, n2, n3 = (int(v) for v in dims[1:].split("x"))
        x = engine_mod.corr_rand_3d(n1, n2, n3, float(xi[2:]), int(s[1:]), bool(int(u[1:])),
                                    float(m[1:])).reshape(-1)
        stride = int(g[name + "__stride"][0])
        np.testing.assert_allclose(x[::stride], g[k], rtol=0, atol=1e-12)
        n += 1
    assert n >= 5


def test_vacancies_and_spins_match_oracle(engine_mod, oracle):
    for mode, pp in [(0, 0.05), (0, 0.3), (1, 0.1)]:
        a = engine_mod.setup_vacancies(17, 8, 6, pp, 0.1, 0.2, mode)
        b = oracle.setup_vacancies(17, 8, 6, pp, 0.1, 0.2, mode)
        for x, y in zip(a[:3], b[:3]):
            np.testing.assert_array_equal(x, y)
        assert a[3] == b[3]
    for start in (0, 1, 2):
        for axis in (0, 1):
            np.testing.assert_array_equal(engine_mod.kiss_spins(5, 6, 4, start, axis),
                                          oracle.init_spins(5, 6, 4, start, axis))


def test_ladder_matches_oracle(engine_mod, oracle):
    for n in (1, 2, 16, 32):
        np.testing.assert_array_equal(engine_mod.ladder(n, 8.0, 11.5), oracle.ladder(n, 8.0, 11.5))
    np.testing.assert_array_equal(engine_mod.ladder(11, 8.0, 11.5, True, 9.5, 0.7),
                                  oracle.ladder(11, 8.0, 11.5, True, 9.5, 0.7))


def test_argument_validation_without_gpu(engine_mod):
    with pytest.raises(engine_mod.J1J2CError) as e:
        engine_mod.Engine(7, 8)  # odd L (8-colour update needs even L)
    assert e.value.code == engine_mod.EINVAL
    with pytest.raises(engine_mod.J1J2CError):
        engine_mod.Engine(8, 8, ptswapever=0)
    with pytest.raises(engine_mod.J1J2CError):
        engine_mod.Engine(8, 8, precision=7)
    with pytest.raises(engine_mod.J1J2CError):
        engine_mod.ladder(4, 9.0, 8.0)
