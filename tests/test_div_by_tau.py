"""The synapse decay's division without a hardware divide (div_by_tau in
eden_gb300/csrc/eden_kernels.cuh): q = RN(x*r), e = fma(-q, tau, x),
RN(q + r*e) with r = RN(1/tau), and hardware division below 2^-100.
This restates the same IEEE single-precision operations on the CPU (libm's
fmaf is the correctly rounded fused multiply-add the GPU's FFMA also is)
and checks the result equals the correctly rounded quotient x / tau for the
synapse time constants in use and operands across the whole normal range."""
import ctypes
import ctypes.util

import numpy as np
import pytest

libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
libm.fmaf.restype = ctypes.c_float
libm.fmaf.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float]
F = np.float32


def div_by_tau(x, tau, r):
    if abs(x) < F(2.0 ** -100):
        return F(x / tau)
    q = F(x * r)
    e = F(libm.fmaf(-q, tau, x))
    return F(libm.fmaf(e, r, q))


@pytest.mark.parametrize("tau", [500.0, 2000.0, 5000.0, 123.456, 7.0, 37.5, 1.0e4])
def test_matches_correctly_rounded_quotient(tau):
    rng = np.random.default_rng(7)
    tau = F(tau)
    r = F(F(1.0) / tau)
    # magnitudes from 2^-99 to 2^10, both signs, plus values near powers of two
    mags = np.exp2(rng.uniform(-99, 10, 20000)).astype(F)
    xs = np.concatenate([mags, -mags, np.exp2(np.arange(-99, 10)).astype(F)])
    bad = [float(x) for x in xs if div_by_tau(F(x), tau, r) != F(F(x) / tau)]
    assert not bad, f"{len(bad)} mismatches, e.g. {bad[:3]}"
