"""ORACLE — test infrastructure only.

numpy restatement of make_corr_rand_3d (sim/corr_rand_3d.f90:191-386): exponential correlation
on the power-of-two padded periodic cube (CR:235-268, CR:362-384), KISS polar-method Gaussian
noise in Fortran order after gkissinit(seed) (CR:256, CR:280-287), Fourier filter
Xk * sqrt(|Re Ck|) (CR:303-310), inverse transform and crop (CR:315-328), and the erfcc map to
uniform [-max_value, max_value] (CR:333-341).

Ooura's RDFT uses exp(+i...) where numpy uses exp(-i...); the filter is real and even, so the
filtered inverse transform is the same field either way (checked against the Ooura-linked build
in tests/golden/).
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O


def nextpow2(n: int) -> int:
    p = 1
    while p < n:
        p *= 2
    return p


def corr_cube(f1: int, f2: int, f3: int, xi: float) -> np.ndarray:
    """C(dx,dy,dz) on the padded cube, array[k, j, i] (i fastest, as the Fortran loop)."""
    i = np.arange(f1)
    j = np.arange(f2)
    k = np.arange(f3)
    dx = np.minimum(i, f1 - i)
    dy = np.minimum(j, f2 - j)
    dz = np.minimum(k, f3 - k)
    r2 = dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2
    r = np.sqrt(r2.astype(np.float64))
    if xi <= 0.0:
        return (r == 0.0).astype(np.float64)
    return np.exp(-r / xi)


def make_corr_rand_3d(n1, n2, n3, xi, seed, do_uniform=True, max_value=2.0) -> np.ndarray:
    f1, f2, f3 = nextpow2(n1), nextpow2(n2), nextpow2(n3)
    c = corr_cube(f1, f2, f3, xi)
    ck = np.fft.rfftn(c)
    noise = O.gkiss_fill(seed, f1 * f2 * f3).reshape(f3, f2, f1)
    xk = np.fft.rfftn(noise)
    xk *= np.sqrt(np.abs(ck.real))
    x = np.fft.irfftn(xk, s=(f3, f2, f1), axes=(0, 1, 2))[:n3, :n2, :n1]
    if do_uniform:
        erf = np.vectorize(O.erfcc)
        x = (2.0 * (1.0 - 0.5 * erf(x / math.sqrt(2.0))) - 1.0) * max_value
    return np.ascontiguousarray(x)
