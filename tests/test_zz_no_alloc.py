"""GPU test of j1j2c_enumerate_exact_noalloc, the allocation-free exact enumeration for callers
that cannot allocate device memory when they need it (their memory pool already holds the GPU,
or the calling loop must not pay for an allocation).  Its results must equal those of the
allocating entry point j1j2c_enumerate_exact on the same inputs, on consecutive calls that share
its fixed scratch array, and it must refuse requests beyond that array's capacity.

Collected last on purpose (file name), so that a run stopping at the first failure has already
run every other test; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(jc, fn, L, H, p, betas, occu=None):
    p = np.ascontiguousarray(p, np.float64)
    b = np.ascontiguousarray(betas, np.float64)
    out = np.full((b.size, 12), np.nan)
    o = None if occu is None else np.ascontiguousarray(occu, np.int8)
    rc = fn(C.c_int32(L), C.c_int32(H), C.c_double(1.0), C.c_double(1.0), C.c_double(-1.0),
            C.c_double(1.0), p.ctypes.data_as(C.POINTER(C.c_double)),
            None if o is None else o.ctypes.data_as(C.POINTER(C.c_int8)), None, None,
            C.c_int32(b.size), b.ctypes.data_as(C.POINTER(C.c_double)),
            out.ctypes.data_as(C.POINTER(C.c_double)))
    return rc, out


def test_noalloc_enumeration_matches_allocating_entry_point(engine_mod):
    jc = engine_mod
    lib = jc.lib()
    cases = [
        (4, 2, jc.disorder(4, 2, 5), [1 / 6.0, 1 / 8.0, 1 / 10.0, 1 / 12.0], None),  # 512 CTAs
        (2, 4, jc.disorder(2, 4, 7), [0.05, 0.2, 0.4], [1] * 15 + [0]),            # 1 CTA, after
    ]
    for L, H, p, betas, occu in cases:  # two calls in a row on the shared scratch array
        rc_ref, ref = _call(jc, lib.j1j2c_enumerate_exact, L, H, p, betas, occu)
        assert rc_ref == 0, lib.j1j2c_last_error(None)
        rc, got = _call(jc, lib.j1j2c_enumerate_exact_noalloc, L, H, p, betas, occu)
        assert rc == 0, lib.j1j2c_last_error(None)
        np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-11)


def test_noalloc_enumeration_rejects_oversize_requests(engine_mod):
    jc = engine_mod
    lib = jc.lib()
    rc, _ = _call(jc, lib.j1j2c_enumerate_exact_noalloc, 4, 4, np.zeros(64), [0.1])
    assert rc == jc.EINVAL and b"32 sites" in lib.j1j2c_last_error(None)
    rc, _ = _call(jc, lib.j1j2c_enumerate_exact_noalloc, 2, 2, np.zeros(8), [0.1] * 5)
    assert rc == jc.EINVAL
