// Device-side arithmetic of the simulation step, shared by the per-step and
// the windowed kernels.  Every expression keeps the operation order of the
// reference's generated C so single-precision results stay within rounding
// of it (the reference compiles with -Ofast, so bit equality is not defined).
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

#include "../../include/eden_gpu.h"

namespace eden {

// Thomas Wang's 64-bit integer hash (eden/Eden.cpp:3199-3213).
__device__ __forceinline__ uint64_t hash64shift(uint64_t key) {
    key = (~key) + (key << 21);
    key = key ^ (key >> 24);
    key = (key + (key << 3)) + (key << 8);
    key = key ^ (key >> 14);
    key = (key + (key << 2)) + (key << 4);
    key = key ^ (key >> 28);
    key = key + (key << 31);
    return key;
}

// randof(x, work_item, instance, step, invocation) (eden/Eden.cpp:3216-3233):
// 24 bits of instance, 40 bits of step, hashed 128 -> 64 bits, 23-bit mantissa.
__device__ __forceinline__ float randof(float x, int64_t work_item, int64_t instance, int64_t step,
                                        int invocation_id) {
    uint64_t hi = ((uint64_t)work_item << 24) | ((uint64_t)instance & ((1ULL << 24) - 1));
    uint64_t lo = ((uint64_t)(int64_t)invocation_id << 40) | ((uint64_t)step & ((1ULL << 40) - 1));
    uint64_t sample = hash64shift(hash64shift(lo) ^ hi);
    const int scale = 1 << 23;
    float r = (float)(uint32_t)(sample & (uint64_t)(scale - 1)) / (float)scale;
    return x * r;
}

// HH rate forms (eden/Eden.cpp:5164-5181), evaluated without branching on
// the form so that the gates of a warp with different forms do not diverge;
// each form keeps its own operations: EXP r * exp(x), EXPLINEAR
// r * (x / (1 - exp(-x))) (r where V == mid), SIGMOID r / (1 + exp(-x)),
// with x = (V - mid) / s (mid - V is exactly -(V - mid)).
__device__ __forceinline__ float rate_value(int kind, float r, float mid, float s, float v) {
    const float x = (v - mid) / s;
    const float e = expf(kind == EDEN_RATE_EXP ? x : -x);
    const bool sig = kind == EDEN_RATE_SIGMOID;
    const float q = (sig ? r : x) / (sig ? 1.0f + e : 1.0f - e);
    if (kind == EDEN_RATE_EXP) return r * e;
    if (sig) return q;
    return r * ((v == mid) ? 1.0f : q);
}

// One HH gate for one step (eden/Eden.cpp:5126-5259): exponential-Euler
// relaxation towards inf(V) with time constant tau(V), clamped to
// [1e-6, 1 - 1e-6]; initialisation sets it to inf(V).
__device__ __forceinline__ float gate_relax_ti(float tau, float inf, float q10, bool init, float dt, float qo) {
    if (init) return inf;
    const float blend = expf(-((dt * q10) / tau));
    float qn = blend * qo + (1.0f - blend) * inf;
    if (!(qn > 1e-6f)) qn = 1e-6f;
    if (!(qn < (float)(1 - 1e-6))) qn = (float)(1 - 1e-6);
    return qn;
}

// A gate from its forward and reverse rates: tau = 1 / (a + b), inf = a / (a + b).
__device__ __forceinline__ float gate_relax(float alpha, float beta, float q10, bool init, float dt, float qo) {
    return gate_relax_ti(1.0f / (alpha + beta), alpha / (alpha + beta), q10, init, dt, qo);
}

// A timeCourse / steadyState form: a rate form, or a constant (fixedTimeCourse).
__device__ __forceinline__ float form_value(int kind, float r, float mid, float s, float v) {
    return kind == EDEN_RATE_FIXED ? r : rate_value(kind, r, mid, s, v);
}

// A gate of any kind (eden/Eden.cpp:5290-5375): tau and inf from its own
// timeCourse / steadyState where the kind has them, else from the rates.
__device__ __forceinline__ float gate_general(int gk, int fk, float fr, float fm, float fs, int rk, float rr, float rm,
                                              float rs, int tk, float tr, float tm, float ts, int ik, float ir,
                                              float im, float is, float q10, bool init, float dt, float v, float qo) {
    if (gk == EDEN_GATE_INSTANTANEOUS) return form_value(ik, ir, im, is, v);
    float a = 0.0f, b = 0.0f;
    if (gk != EDEN_GATE_TAUINF) {
        a = rate_value(fk, fr, fm, fs, v);
        b = rate_value(rk, rr, rm, rs, v);
    }
    const bool own_tau = gk == EDEN_GATE_TAUINF || gk == EDEN_GATE_RATESTAU || gk == EDEN_GATE_RATESTAUINF;
    const bool own_inf = gk == EDEN_GATE_TAUINF || gk == EDEN_GATE_RATESINF || gk == EDEN_GATE_RATESTAUINF;
    const float tau = own_tau ? form_value(tk, tr, tm, ts, v) : 1.0f / (a + b);
    const float inf = own_inf ? form_value(ik, ir, im, is, v) : a / (a + b);
    return gate_relax_ti(tau, inf, q10, init, dt, qo);
}

// Channel type table in constant memory (a handful of ionChannelHH types).
constexpr int kMaxChanTypes = 32;
constexpr int kMaxSynTypes = 32;

}  // namespace eden
