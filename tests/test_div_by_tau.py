"""The synapse decay's division without a hardware divide (div_by_tau in
eden_gb300/csrc/eden_kernels.cuh): q = RN(x*r), e = fma(-q, tau, x),
RN(q + r*e) with r = RN(1/tau), operands below 2^-100 scaled by 2^64
before and the quotient by 2^-64 after.
This restates the same IEEE single-precision operations on the CPU (libm's
fmaf is the correctly rounded fused multiply-add the GPU's FFMA also is)
and checks the result equals the correctly rounded quotient x / tau for the
synapse time constants in use and operands across the whole normal range,
and to within one subnormal ulp (2^-149) for tiny and subnormal operands."""
import ctypes
import ctypes.util

import numpy as np
import pytest

libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
libm.fmaf.restype = ctypes.c_float
libm.fmaf.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float]
F = np.float32


def div_by_tau(x, tau, r):
    tiny = abs(x) < F(2.0 ** -100)
    xs = F(x * F(2.0 ** 64)) if tiny else x
    q = F(xs * r)
    e = F(libm.fmaf(-q, tau, xs))
    qs = F(libm.fmaf(e, r, q))
    return F(qs * F(2.0 ** -64)) if tiny else qs


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


@pytest.mark.parametrize("tau", [500.0, 5000.0, 2000.0, 7.0])
def test_tiny_and_subnormal_operands(tau):
    rng = np.random.default_rng(11)
    tau = F(tau)
    r = F(F(1.0) / tau)
    with np.errstate(under="ignore"):
        mags = np.exp2(rng.uniform(-149, -99, 20000)).astype(F)
        xs = np.concatenate([mags, -mags, np.exp2(np.arange(-149, -99)).astype(F), [F(0.0)]])
        for x in xs:
            got, want = div_by_tau(F(x), tau, r), F(F(x) / tau)
            if abs(want) >= F(2.0 ** -126):
                assert got == want, (float(x), float(got), float(want))
            else:
                assert abs(float(got) - float(want)) <= 2.0 ** -149, (float(x), float(got), float(want))
