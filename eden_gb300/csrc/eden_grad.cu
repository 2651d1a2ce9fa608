// Gradients of recorded membrane potentials with respect to channel
// conductivities and cell axial resistivities (include/eden_gpu.h,
// edenGpuGrad*).  The reference has no gradient path; this file has no
// counterpart there.
//
// The forward step is the one the reference runs per compartment and the
// plain GPU path reproduces: HH gates by exponential Euler with clamp
// (eden/Eden.cpp:5126-5259), channel currents (5805-5898), the V pre-update
// (6057-6107) and the backward-Euler Hines solve (6114-6225).  The gradient
// is the discrete adjoint of that step (reverse mode, exact for the
// arithmetic of the step up to rounding):
//
//   state (V^n, q^n) -> q^{n+1} = Q(V^n, q^n)            (gates, old V)
//                       g_c = gbase_c fopen_c(q^n) 1e-5 A  (channel conductance)
//                       d = G/C + s irc,  x = V + dt (I + V G)/C
//                       M V^{n+1} = x,  M = 1 + dt d on the diagonal,
//                                      s U (row child), s L (row parent)
//   with s = Ra_ref / Ra the cell's axial scale.  Given the adjoints
//   (lV, lq) of (V^{n+1}, q^{n+1}):  mu = M^-T lV (the same elimination with
//   U and L exchanged), x_bar = mu, d_bar = -dt mu V^{n+1};
//   g_bar_c = (d_bar + mu dt E_c) / C; Ra_bar += (1/Ra) mu^T A_ax V^{n+1}
//   (A_ax the axial part of M); V_bar = x_bar + sum lq dQ/dV; q_bar = lq
//   dQ/dq + g_bar gbase 1e-5 A dfopen/dq.  dQ/dq = b and dQ/dV = b'(q - inf)
//   + (1 - b) inf' where the gate did not clamp, 0 where it did.
//
// Synaptic drive with event steps fixed in advance -- timedSynapticInput
// inputs and connection synapses whose presynaptic cell is a spike source
// (spike lists, generators, event-set readers) -- enters each step as
// conductances g_k = sum_s w_s g^_s(n) per group k (one compartment, one
// synapse type, inputs or connections), with g^_s the unit-weight exposure
// of synapse s at step n (expTwo gbase (B - A), expOne G;
// LEMS_CoreComponents.inc.xml:145-180, eden/Eden.cpp:3424-3466): forward
// Euler between events, the event's jump instead of the decay in its step.
// g^_s does not depend on V or on the weights, so a k_grad_drive launch
// tabulates g_k(n) for the run before the forward, and the adjoint gives
// g_bar_k(n) = (d_bar + mu dt E_k) / C like a channel's; a weight's gradient
// is then sum_n g_bar_k(n) g^_s(n) (eden/Eden.cpp:3708-3710 multiplies the
// synapse's current and conductance by its weight), summed per synapse in
// double by k_grad_weights.
//
// Cells are independent, so one warp carries one cell through the whole run
// in one launch, synchronising only within the warp.  The forward kernel
// writes the trace and a checkpoint of (V, q) every S steps; the backward
// kernel walks the segments last to first, recomputes each from its
// checkpoint into a trajectory buffer and runs the adjoint steps back
// through it.  Parameter contributions accumulate per lane in double, in a
// fixed order, and are summed per cell and then per parameter in a fixed
// order, so gradients are deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/eden_gpu.h"
#include "eden_math.cuh"

using namespace eden;

namespace eden_grad {

constexpr int kMaxSlots = 32;  // distinct parameters one cell may use

// A synapse type as the drive needs it: kind, gbase (uS), time constants
// (us) and expTwo's jump weight_prop * waveform_factor.
struct GradSyn {
    int32_t kind;
    float gbase, tau_decay, tau_rise, wf_w;
};

struct GradDev {
    int n_cells = 0, n_rec = 0, S = 100, n_types = 0;
    int64_t N = 0, n_comp = 0, n_gate = 0;
    float dt = 0.0f;
    // per cell: compartments, gates, channels, depth table, parameter slots, recorded columns
    const int32_t *cell_c0, *cell_g0, *cell_ch0, *cell_l0, *cell_s0, *cell_r0;
    const int32_t *cell_ra_slot, *cell_ra_param, *cell_chain;
    const float *cell_ra;
    const int32_t *lev;  // each cell's depth boundaries (local indices), nlev + 1 entries
    // per compartment, breadth-first within the cell
    const float *C, *A, *IRC, *U, *L, *V0;
    const int32_t *P, *CB, *CE, *comp_ch0, *comp_pu0;  // local indices; comp_ch0 local to the cell
    // per channel instance
    const int32_t *ch_type, *ch_g0, *ch_param, *ch_slot;
    const float *ch_gbase, *ch_erev;
    const EdenGpuChannelType *types;
    // pulses
    const float *pu_start, *pu_dur, *pu_aw;
    // recorded compartments (local index) and their trace columns
    const int32_t *rec_local, *rec_col;
    const float *tk;  // [N + 1]: tk[n] = time of step n
    // synaptic drive: groups of each compartment (breadth-first order),
    // each group's reversal potential, kind (0 inputs, 1 connections) and
    // items; each item's synapse type, weight (or parameter) and event steps
    int32_t n_grp = 0;
    int64_t n_item = 0;
    const int32_t *comp_gr0, *gr_kind, *gr_it0, *it_grp, *it_type, *it_param, *it_ev;
    const int64_t *it_ev0;
    const float *gr_erev, *it_w;
    const GradSyn *syn;
    float *it_a, *it_b;      // unit-weight synapse state while tabulating
    int64_t *it_cur;         // its next event
    float *gtab;             // [N + 1][n_grp] group conductance at step n (weights applied)
    float *gbar;             // [N + 1][n_grp] its adjoint
    double *item_grad;       // [n_item] d loss / d weight
    const float *params;
    float *ck_v, *ck_q;  // checkpoints [n_ck][n_comp], [n_ck][n_gate]
    float *tr_v, *tr_q;  // one segment's trajectory [S + 1][n_comp], [S + 1][n_gate]
    float *trace;        // [N][n_rec]
    const float *trace_grad;
    double *slot_grad;   // per cell and slot
};

// Largest cell, for the shared-memory layout.
struct Dims {
    int slots, c, g, ch;
};

// One warp's shared memory: parameter accumulators, the channel types, the
// cell's state and solve arrays, and its constants staged once per launch
// (axial terms already scaled by the cell's resistivity parameter).
struct Cell {
    double *acc;  // [slots][32]
    EdenGpuChannelType *types;
    float *V, *VN, *X, *D, *LV, *q, *LQ;
    float *Us, *Ls, *Cc, *Ac, *IRCs;
    int32_t *P, *CB, *CE, *ch0;
    int32_t *ctype, *cg0, *cslot;
    float *cgb, *cerev;
    int c0, g0, nc, ng, nch, nlev, ra_slot;
    const int32_t *lev;
    bool serial;  // solve by one lane (cells with few compartments per depth)
    bool chain;   // an unbranched cable: node j's only child is j + 1
};

__device__ __forceinline__ Cell stage_cell(const GradDev &m, int cell, const Dims &dm) {
    extern __shared__ double smem_d[];
    const int lane = threadIdx.x & 31;
    Cell c;
    c.acc = smem_d;
    c.types = reinterpret_cast<EdenGpuChannelType *>(smem_d + (size_t)dm.slots * 32);
    float *f = reinterpret_cast<float *>(c.types + m.n_types);
    c.V = f; f += dm.c;
    c.VN = f; f += dm.c;
    c.X = f; f += dm.c;
    c.D = f; f += dm.c;
    c.LV = f; f += dm.c;
    c.Us = f; f += dm.c;
    c.Ls = f; f += dm.c;
    c.Cc = f; f += dm.c;
    c.Ac = f; f += dm.c;
    c.IRCs = f; f += dm.c;
    c.q = f; f += dm.g;
    c.LQ = f; f += dm.g;
    c.cgb = f; f += dm.ch;
    c.cerev = f; f += dm.ch;
    int32_t *i = reinterpret_cast<int32_t *>(f);
    c.P = i; i += dm.c;
    c.CB = i; i += dm.c;
    c.CE = i; i += dm.c;
    c.ch0 = i; i += dm.c + 1;
    c.ctype = i; i += dm.ch;
    c.cg0 = i; i += dm.ch;
    c.cslot = i;
    c.c0 = m.cell_c0[cell];
    c.nc = m.cell_c0[cell + 1] - c.c0;
    c.g0 = m.cell_g0[cell];
    c.ng = m.cell_g0[cell + 1] - c.g0;
    const int h0 = m.cell_ch0[cell];
    c.nch = m.cell_ch0[cell + 1] - h0;
    c.lev = m.lev + m.cell_l0[cell];
    c.nlev = m.cell_l0[cell + 1] - m.cell_l0[cell] - 1;
    c.ra_slot = m.cell_ra_slot[cell];
    c.serial = c.nc <= 6 * c.nlev;
    c.chain = m.cell_chain[cell] != 0;
    const int rp = m.cell_ra_param[cell];
    const float s = rp >= 0 ? m.cell_ra[cell] / m.params[rp] : 1.0f;
    const int words = (int)(sizeof(EdenGpuChannelType) / 4) * m.n_types;
    for (int k = lane; k < words; k += 32)
        reinterpret_cast<int32_t *>(c.types)[k] = reinterpret_cast<const int32_t *>(m.types)[k];
    for (int j = lane; j < c.nc; j += 32) {
        const int gc = c.c0 + j;
        c.Us[j] = m.U[gc] * s;
        c.Ls[j] = m.L[gc] * s;
        c.IRCs[j] = m.IRC[gc] * s;
        c.Cc[j] = m.C[gc];
        c.Ac[j] = m.A[gc];
        c.P[j] = m.P[gc];
        c.CB[j] = m.CB[gc];
        c.CE[j] = m.CE[gc];
        c.ch0[j] = m.comp_ch0[gc];
    }
    if (lane == 0) c.ch0[c.nc] = c.nch;
    for (int k = lane; k < c.nch; k += 32) {
        const int ch = h0 + k;
        const int p = m.ch_param[ch];
        c.ctype[k] = m.ch_type[ch];
        c.cg0[k] = m.ch_g0[ch];
        c.cslot[k] = m.ch_slot[ch];
        c.cgb[k] = p >= 0 ? m.params[p] : m.ch_gbase[ch];
        c.cerev[k] = m.ch_erev[ch];
    }
    __syncwarp();
    return c;
}

// d(rate)/dV of the HH rate forms of rate_value, from the mathematics of
// each form: EXP r e^x -> val / s; SIGMOID r / (1 + e^-x) -> val (e^-x / (1 +
// e^-x)) / s; EXPLINEAR r f(x), f = x / (1 - e^-x) -> r f'(x) / s with
// f'(x) = (1 - e^-x (1 + x)) / (1 - e^-x)^2, by its Taylor series
// 1/2 + x/6 - x^3/180 near x = 0 (where the closed form cancels).
__device__ __forceinline__ float rate_slope(int kind, float r, float mid, float s, float v, float val) {
    const float x = (v - mid) / s;
    if (kind == EDEN_RATE_EXP) return val / s;
    if (kind == EDEN_RATE_SIGMOID) {
        const float e = expf(-x);
        return val * (1.0f / (1.0f + 1.0f / e)) / s;
    }
    float fp;
    if (fabsf(x) < 1e-2f) {
        fp = 0.5f + x * (1.0f / 6.0f) - x * x * x * (1.0f / 180.0f);
    } else if (x < -60.0f) {
        fp = 0.0f;
    } else {
        const float em = expm1f(-x);  // e^-x - 1
        fp = (-em - x * (1.0f + em)) / (em * em);
    }
    return r * fp / s;
}

// Channels and V pre-update of compartment j at time t: advances its gates
// in place and returns the pre-updated V (x) and the diagonal term d, with
// the plain path's operations (target_step).
__device__ __forceinline__ void comp_pre(const GradDev &m, const Cell &c, int j, int64_t n, float t, float v,
                                         bool init, float &x, float &d) {
    const float A = c.Ac[j];
    float Ich = 0.0f, Gch = 0.0f;
    for (int k = c.ch0[j]; k < c.ch0[j + 1]; k++) {
        const EdenGpuChannelType &ct = c.types[c.ctype[k]];
        float *qq = c.q + c.cg0[k];
        float fopen = 1.0f;
        for (int g = 0; g < ct.n_gates; g++) {
            const float qo = qq[g];
            const float al = rate_value(ct.fwd_kind[g], ct.fwd_rate[g], ct.fwd_mid[g], ct.fwd_scale[g], v);
            const float be = rate_value(ct.rev_kind[g], ct.rev_rate[g], ct.rev_mid[g], ct.rev_scale[g], v);
            qq[g] = gate_relax(al, be, ct.q10[g], init, m.dt, qo);
            for (int r = 0; r < ct.gate_instances[g]; r++) fopen = fopen * qo;
        }
        const float gs = c.cgb[k] * fopen;
        Ich += (gs * (c.cerev[k] - v) * 1e-5f) * A;
        Gch += (gs * 1e-5f) * A;
    }
    float Iin = 0.0f;
    const int gc = c.c0 + j;
    for (int k = m.comp_pu0[gc]; k < m.comp_pu0[gc + 1]; k++) {
        const float st = m.pu_start[k], du = m.pu_dur[k];
        Iin += (st <= t && t <= st + du) ? m.pu_aw[k] : 0.0f;
    }
    // synaptic drive: inputs, then connections (eden/Eden.cpp:6057-6060)
    float Gin = 0.0f, Isyn = 0.0f, Gsyn = 0.0f;
    if (!init)
        for (int k = m.comp_gr0[gc]; k < m.comp_gr0[gc + 1]; k++) {
            const float g = m.gtab[n * m.n_grp + k];
            if (m.gr_kind[k] == 0) {
                Iin += g * (m.gr_erev[k] - v);
                Gin += g;
            } else {
                Isyn += g * (m.gr_erev[k] - v);
                Gsyn += g;
            }
        }
    const float I = Ich + Iin + Isyn;
    const float G = Gch + Gin + Gsyn;
    const float C = c.Cc[j];
    d = 1.0f * (G / C) + c.IRCs[j];
    x = init ? v : v + (m.dt * (I + (v * G))) / C;
}

// The total conductance of compartment gc at step n, its channels' Gch
// plus its drive groups', summed in comp_pre's order.
__device__ __forceinline__ float total_g(const GradDev &m, int gc, int64_t n, float Gch) {
    float Gin = 0.0f, Gsyn = 0.0f;
    for (int k = m.comp_gr0[gc]; k < m.comp_gr0[gc + 1]; k++) {
        const float g = m.gtab[n * m.n_grp + k];
        if (m.gr_kind[k] == 0) Gin += g;
        else Gsyn += g;
    }
    return Gch + Gin + Gsyn;
}

// Backward-Euler Hines solve of the cell (eden/Eden.cpp:6114-6225): D holds
// the diagonal terms on entry and the reciprocal pivots on return, X the
// pre-updated V on entry and V_next on return; every node pulls its children
// in order, deepest first, then back-substitution runs root first.  With
// `transposed` it solves M^T y = X: the same pivots, the right-hand side
// eliminated with U and back-substituted with L.  Cells with few
// compartments per depth (chains, ball-and-stick) are solved by one lane in
// reverse breadth-first order with the last node's values in registers; the
// others depth by depth across the warp.  Both do the same operations.
__device__ __forceinline__ void hines_cell(float dt, const Cell &c, bool transposed) {
    const int lane = threadIdx.x & 31;
    float *D = c.D, *X = c.X;
    if (c.chain) {
        // the same operations with every value of the previous node in registers
        if (lane == 0) {
            const int n = c.nc;
            float rc = __fdividef(1.0f, 1.0f + D[n - 1] * dt);
            float xc = X[n - 1];
            D[n - 1] = rc;
#pragma unroll 4
            for (int j = n - 2; j >= 0; j--) {
                const float Ui = c.Us[j + 1];
                const float ratio = c.Ls[j + 1] * rc;
                float dj = 1.0f + D[j] * dt;
                dj -= ratio * Ui;
                const float xj = X[j] - (transposed ? Ui * rc : ratio) * xc;
                X[j] = xj;
                rc = __fdividef(1.0f, dj);
                D[j] = rc;
                xc = xj;
            }
            float xp = X[0] * D[0];
            X[0] = xp;
#pragma unroll 4
            for (int j = 1; j < n; j++) {
                const float off = transposed ? c.Ls[j] : c.Us[j];
                xp = (X[j] - off * xp) * D[j];
                X[j] = xp;
            }
        }
        __syncwarp();
        return;
    }
    if (c.serial) {
        if (lane == 0) {
            float xc = 0.0f, rc = 0.0f;
            int last = -1;
            for (int j = c.nc - 1; j >= 0; j--) {
                const int kb = c.CB[j], ke = c.CE[j];
                float dj = 1.0f + D[j] * dt;
                float xj = X[j];
                if (ke > kb) {
                    for (int i = kb; i < ke; i++) {
                        const float xi = i == last ? xc : X[i];
                        const float ri = i == last ? rc : D[i];
                        const float Ui = c.Us[i];
                        const float ratio = c.Ls[i] * ri;
                        dj -= ratio * Ui;
                        xj -= (transposed ? Ui * ri : ratio) * xi;
                    }
                    X[j] = xj;
                }
                rc = __fdividef(1.0f, dj);
                D[j] = rc;
                xc = xj;
                last = j;
            }
            float xp = X[0] * D[0];
            X[0] = xp;
            for (int j = 1; j < c.nc; j++) {
                const int p = c.P[j];
                const float off = transposed ? c.Ls[j] : c.Us[j];
                const float xpar = p == j - 1 ? xp : X[p];
                xp = (X[j] - off * xpar) * D[j];
                X[j] = xp;
            }
        }
        __syncwarp();
        return;
    }
    for (int j = lane; j < c.nc; j += 32) D[j] = 1.0f + D[j] * dt;
    __syncwarp();
    for (int l = c.nlev - 1; l >= 0; l--) {
        for (int j = c.lev[l] + lane; j < c.lev[l + 1]; j += 32) {
            const int kb = c.CB[j], ke = c.CE[j];
            float dj = D[j];
            if (ke > kb) {
                float xj = X[j];
                for (int i = kb; i < ke; i++) {
                    const float Ui = c.Us[i];
                    const float ratio = c.Ls[i] * D[i];
                    dj -= ratio * Ui;
                    xj -= (transposed ? Ui * D[i] : ratio) * X[i];
                }
                X[j] = xj;
            }
            D[j] = __fdividef(1.0f, dj);
        }
        __syncwarp();
    }
    for (int r = c.lev[0] + lane; r < c.lev[1]; r += 32) X[r] = X[r] * D[r];
    __syncwarp();
    for (int l = 1; l < c.nlev; l++) {
        for (int i = c.lev[l] + lane; i < c.lev[l + 1]; i += 32) {
            const float off = transposed ? c.Ls[i] : c.Us[i];
            X[i] = (X[i] - off * X[c.P[i]]) * D[i];
        }
        __syncwarp();
    }
}

// One forward step n -> n + 1 of the staged cell.
__device__ __forceinline__ void forward_step(const GradDev &m, const Cell &c, int64_t n) {
    const int lane = threadIdx.x & 31;
    const float t = m.tk[n];
    for (int j = lane; j < c.nc; j += 32) {
        float x, d;
        comp_pre(m, c, j, n, t, c.V[j], false, x, d);
        c.X[j] = x;
        c.D[j] = d;
    }
    __syncwarp();
    hines_cell(m.dt, c, false);
    for (int j = lane; j < c.nc; j += 32) c.V[j] = c.X[j];
    __syncwarp();
}

__global__ void __launch_bounds__(32) k_grad_forward(GradDev m, Dims dm) {
    const int cell = blockIdx.x, lane = threadIdx.x;
    const Cell c = stage_cell(m, cell, dm);
    for (int j = lane; j < c.nc; j += 32) c.V[j] = m.V0[c.c0 + j];
    for (int k = lane; k < c.ng; k += 32) c.q[k] = 0.0f;
    __syncwarp();
    // the four initialisation passes leave V and set every gate to inf(V)
    for (int j = lane; j < c.nc; j += 32) {
        float x, d;
        comp_pre(m, c, j, 0, 0.0f, c.V[j], true, x, d);
    }
    const int r0 = m.cell_r0[cell], r1 = m.cell_r0[cell + 1];
    int64_t ck = 0;
    int to_ck = 0;  // steps until the next checkpoint
    for (int64_t n = 1; n <= m.N; n++) {
        __syncwarp();
        if (to_ck == 0 && n < m.N) {
            for (int j = lane; j < c.nc; j += 32) m.ck_v[ck * m.n_comp + c.c0 + j] = c.V[j];
            for (int k = lane; k < c.ng; k += 32) m.ck_q[ck * m.n_gate + c.g0 + k] = c.q[k];
            ck++;
            to_ck = m.S;
        }
        to_ck--;
        for (int r = r0 + lane; r < r1; r += 32) m.trace[(n - 1) * m.n_rec + m.rec_col[r]] = c.V[m.rec_local[r]];
        if (n < m.N) forward_step(m, c, n);
    }
}

// lV += the trace gradient of step n (one lane: recorded columns may share
// a compartment).
__device__ __forceinline__ void add_trace_grad(const GradDev &m, int cell, int64_t n, float *LV) {
    if ((threadIdx.x & 31) == 0)
        for (int r = m.cell_r0[cell]; r < m.cell_r0[cell + 1]; r++)
            LV[m.rec_local[r]] += m.trace_grad[(n - 1) * m.n_rec + m.rec_col[r]];
    __syncwarp();
}

// Adjoint of step n -> n + 1: on entry V = V^n, VN = V^{n+1}, q = q^n, LV and
// LQ the adjoints of V^{n+1} and q^{n+1}; on return LV and LQ are those of
// V^n and q^n, and the parameter terms of the step are in acc.
__device__ __forceinline__ void adjoint_step(const GradDev &m, const Cell &c, int64_t n) {
    const int lane = threadIdx.x & 31;
    const float dt = m.dt;
    for (int j = lane; j < c.nc; j += 32) {
        const float A = c.Ac[j];
        float Gch = 0.0f;
        for (int k = c.ch0[j]; k < c.ch0[j + 1]; k++) {
            const EdenGpuChannelType &ct = c.types[c.ctype[k]];
            const float *qq = c.q + c.cg0[k];
            float fopen = 1.0f;
            for (int g = 0; g < ct.n_gates; g++)
                for (int r = 0; r < ct.gate_instances[g]; r++) fopen = fopen * qq[g];
            Gch += ((c.cgb[k] * fopen) * 1e-5f) * A;
        }
        const float G = m.n_grp ? total_g(m, c.c0 + j, n, Gch) : Gch;
        c.D[j] = 1.0f * (G / c.Cc[j]) + c.IRCs[j];
        c.X[j] = c.LV[j];
    }
    __syncwarp();
    hines_cell(dt, c, true);  // X = mu
    double *acc = c.acc + lane;
    for (int j = lane; j < c.nc; j += 32) {
        const float mu = c.X[j], v = c.V[j], vn = c.VN[j];
        const float dbar = -dt * mu * vn;
        float vbar = mu;
        if (c.ra_slot >= 0) {
            double r = (double)mu * (double)(dt * c.IRCs[j]) * vn;
            const int p = c.P[j];
            if (p >= 0) r += (double)mu * (double)c.Us[j] * c.VN[p] + (double)c.X[p] * (double)c.Ls[j] * vn;
            acc[c.ra_slot * 32] += r;
        }
        const float C = c.Cc[j], A = c.Ac[j];
        // the drive groups' conductance adjoints, for the weight gradients
        for (int k = m.comp_gr0[c.c0 + j]; k < m.comp_gr0[c.c0 + j + 1]; k++)
            m.gbar[n * m.n_grp + k] = (dbar + mu * dt * m.gr_erev[k]) / C;
        for (int k = c.ch0[j]; k < c.ch0[j + 1]; k++) {
            const EdenGpuChannelType &ct = c.types[c.ctype[k]];
            const int q0 = c.cg0[k];
            float qo[EDEN_MAX_GATES], pw[EDEN_MAX_GATES];
            float fopen = 1.0f;
#pragma unroll
            for (int g = 0; g < EDEN_MAX_GATES; g++) {
                qo[g] = 1.0f;
                pw[g] = 1.0f;
                if (g < ct.n_gates) {
                    qo[g] = c.q[q0 + g];
                    float p = 1.0f;
                    for (int r = 0; r < ct.gate_instances[g]; r++) p = p * qo[g];
                    pw[g] = p;
                    fopen = fopen * p;
                }
            }
            const float gb = c.cgb[k];
            const float gbar = (dbar + mu * dt * c.cerev[k]) / C;
            const int slot = c.cslot[k];
            if (slot >= 0) acc[slot * 32] += (double)gbar * (double)(fopen * 1e-5f * A);
            const float fbar = gbar * gb * 1e-5f * A;
#pragma unroll
            for (int g = 0; g < EDEN_MAX_GATES; g++) {
                if (g >= ct.n_gates) break;
                // d fopen / d q_g = inst q_g^(inst-1) * prod over the other gates
                const int inst = ct.gate_instances[g];
                float dfdq = 0.0f;
                if (inst > 0) {
                    dfdq = (float)inst;
                    for (int r = 1; r < inst; r++) dfdq = dfdq * qo[g];
#pragma unroll
                    for (int h = 0; h < EDEN_MAX_GATES; h++)
                        if (h != g) dfdq = dfdq * pw[h];
                }
                const float al = rate_value(ct.fwd_kind[g], ct.fwd_rate[g], ct.fwd_mid[g], ct.fwd_scale[g], v);
                const float be = rate_value(ct.rev_kind[g], ct.rev_rate[g], ct.rev_mid[g], ct.rev_scale[g], v);
                const float sum = al + be;
                const float tau = 1.0f / sum;
                const float inf = al / sum;
                const float b = expf(-((dt * ct.q10[g]) / tau));
                const float qn = b * qo[g] + (1.0f - b) * inf;
                const bool clamped = !(qn > 1e-6f) || !(qn < (float)(1 - 1e-6));
                const float lq = c.LQ[q0 + g];
                float qbar = fbar * dfdq;
                if (!clamped) {
                    const float dal = rate_slope(ct.fwd_kind[g], ct.fwd_rate[g], ct.fwd_mid[g], ct.fwd_scale[g], v, al);
                    const float dbe = rate_slope(ct.rev_kind[g], ct.rev_rate[g], ct.rev_mid[g], ct.rev_scale[g], v, be);
                    const float db = -(dt * ct.q10[g]) * (dal + dbe) * b;
                    const float dinf = (dal * be - al * dbe) / (sum * sum);
                    vbar += lq * (db * (qo[g] - inf) + (1.0f - b) * dinf);
                    qbar += lq * b;
                }
                c.LQ[q0 + g] = qbar;
            }
        }
        c.LV[j] = vbar;
    }
    __syncwarp();
}

__global__ void __launch_bounds__(32) k_grad_backward(GradDev m, Dims dm) {
    const int cell = blockIdx.x, lane = threadIdx.x;
    const Cell c = stage_cell(m, cell, dm);
    const int s0 = m.cell_s0[cell], ns = m.cell_s0[cell + 1] - s0;
    for (int k = 0; k < ns; k++) c.acc[k * 32 + lane] = 0.0;
    for (int j = lane; j < c.nc; j += 32) c.LV[j] = 0.0f;
    for (int k = lane; k < c.ng; k += 32) c.LQ[k] = 0.0f;
    __syncwarp();
    add_trace_grad(m, cell, m.N, c.LV);
    const int64_t nseg = m.N >= 2 ? (m.N - 2) / m.S + 1 : 0;
    for (int64_t sg = nseg - 1; sg >= 0; sg--) {
        const int64_t n0 = 1 + sg * m.S, n1 = n0 + m.S < m.N ? n0 + m.S : m.N;
        // recompute the segment's states n0 .. n1 from its checkpoint
        for (int j = lane; j < c.nc; j += 32) {
            const float v = m.ck_v[sg * m.n_comp + c.c0 + j];
            c.V[j] = v;
            m.tr_v[c.c0 + j] = v;
        }
        for (int k = lane; k < c.ng; k += 32) {
            const float q = m.ck_q[sg * m.n_gate + c.g0 + k];
            c.q[k] = q;
            m.tr_q[c.g0 + k] = q;
        }
        __syncwarp();
        for (int64_t n = n0; n < n1; n++) {
            forward_step(m, c, n);
            const int64_t k = n + 1 - n0;
            for (int j = lane; j < c.nc; j += 32) m.tr_v[k * m.n_comp + c.c0 + j] = c.V[j];
            for (int g = lane; g < c.ng; g += 32) m.tr_q[k * m.n_gate + c.g0 + g] = c.q[g];
            __syncwarp();
        }
        // and run the adjoint back through them
        for (int64_t n = n1 - 1; n >= n0; n--) {
            const int64_t k = n - n0;
            for (int j = lane; j < c.nc; j += 32) {
                c.V[j] = m.tr_v[k * m.n_comp + c.c0 + j];
                c.VN[j] = m.tr_v[(k + 1) * m.n_comp + c.c0 + j];
            }
            for (int g = lane; g < c.ng; g += 32) c.q[g] = m.tr_q[k * m.n_gate + c.g0 + g];
            __syncwarp();
            adjoint_step(m, c, n);
            add_trace_grad(m, cell, n, c.LV);
        }
    }
    __syncwarp();
    for (int k = lane; k < ns; k += 32) {
        double tot = 0.0;
        for (int l = 0; l < 32; l++) tot += c.acc[k * 32 + l];
        if (k == c.ra_slot) tot /= (double)m.params[m.cell_ra_param[cell]];
        m.slot_grad[s0 + k] = tot;
    }
}

// The unit-weight exposure of item s at step n and its state update
// (forward Euler; the event's jump instead of the decay in its step).
__device__ __forceinline__ float item_exposure(const GradSyn &st, float a, float b) {
    return st.kind == EDEN_SYN_EXPTWO ? st.gbase * (b - a) : a;
}
__device__ __forceinline__ void item_update(const GradSyn &st, float dt, bool event, float &a, float &b) {
    if (st.kind == EDEN_SYN_EXPTWO) {
        if (event) {
            a = a + st.wf_w;
            b = b + st.wf_w;
        } else {
            a = a + dt * (-a / st.tau_rise);
            b = b + dt * (-b / st.tau_decay);
        }
    } else {
        a = event ? a + st.gbase : a - dt * (a / st.tau_decay);
    }
}

// gtab[n][k] = sum over the group's items of weight * unit-weight exposure,
// for steps 1 .. N - 1 (one thread per group; items in group order).
__global__ void k_grad_drive(GradDev m) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_grp) return;
    const int i0 = m.gr_it0[k], i1 = m.gr_it0[k + 1];
    for (int i = i0; i < i1; i++) {
        m.it_a[i] = 0.0f;
        m.it_b[i] = 0.0f;
        m.it_cur[i] = m.it_ev0[i];
    }
    m.gtab[k] = 0.0f;
    for (int64_t n = 1; n <= m.N; n++) {
        float g = 0.0f;
        for (int i = i0; i < i1; i++) {
            const GradSyn st = m.syn[m.it_type[i]];
            float a = m.it_a[i], b = m.it_b[i];
            const float w = m.it_param[i] >= 0 ? m.params[m.it_param[i]] : m.it_w[i];
            g += w * item_exposure(st, a, b);
            const int64_t e = m.it_cur[i];
            const bool event = e < m.it_ev0[i + 1] && m.it_ev[e] == (int32_t)n;
            if (event) m.it_cur[i] = e + 1;
            item_update(st, m.dt, event, a, b);
            m.it_a[i] = a;
            m.it_b[i] = b;
        }
        m.gtab[n * m.n_grp + k] = g;
    }
}

// d loss / d weight of each item: sum over steps 1 .. N - 1 of the group's
// conductance adjoint times the item's unit-weight exposure, in double.
__global__ void k_grad_weights(GradDev m) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_item) return;
    const int k = m.it_grp[i];
    const GradSyn st = m.syn[m.it_type[i]];
    float a = 0.0f, b = 0.0f;
    int64_t e = m.it_ev0[i];
    const int64_t e1 = m.it_ev0[i + 1];
    double acc = 0.0;
    for (int64_t n = 1; n < m.N; n++) {
        acc += (double)m.gbar[n * m.n_grp + k] * (double)item_exposure(st, a, b);
        const bool event = e < e1 && m.it_ev[e] == (int32_t)n;
        if (event) e++;
        item_update(st, m.dt, event, a, b);
    }
    m.item_grad[i] = acc;
}

}  // namespace eden_grad

using namespace eden_grad;

struct EdenGpuGrad {
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    GradDev d{};
    std::vector<void *> allocs;
    int n_params = 0, n_cells = 0, n_rec = 0;
    Dims dims{1, 1, 1, 1};
    size_t smem = 0;
    std::vector<int32_t> slot_param;     // slot -> parameter
    std::vector<int32_t> cell_ra_param;  // host copy, for the forward's checks
    std::vector<int32_t> item_param;     // parameter that is each drive item's weight, or -1
    std::vector<float> h_params;
    float *d_params = nullptr, *d_trace = nullptr, *d_tgrad = nullptr;
    double *d_slot = nullptr;
    bool have_forward = false;
    double fwd_ms = 0.0, bwd_ms = 0.0;

    int fail(int code, const char *fmt, ...) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
};

#define GTRY(g, call)                                                                               \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return (g)->fail(e_ == cudaErrorMemoryAllocation ? EDEN_GPU_E_NOMEM : EDEN_GPU_E_CUDA,  \
                             "%s failed: %s", #call, cudaGetErrorString(e_));                       \
    } while (0)

namespace {

template <typename T>
int upload(EdenGpuGrad *g, const T **dst, const std::vector<T> &src) {
    void *p = nullptr;
    const size_t bytes = std::max<size_t>(src.size(), 1) * sizeof(T);
    GTRY(g, cudaMalloc(&p, bytes));
    g->allocs.push_back(p);
    if (!src.empty()) GTRY(g, cudaMemcpy(p, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    *dst = static_cast<const T *>(p);
    return 0;
}

template <typename T>
int alloc(EdenGpuGrad *g, T **dst, size_t n) {
    void *p = nullptr;
    GTRY(g, cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    g->allocs.push_back(p);
    *dst = static_cast<T *>(p);
    return 0;
}

bool finite_pos(float x) { return std::isfinite(x) && x > 0.0f; }

int validate(EdenGpuGrad *g, const EdenGpuModel *m, const EdenGpuGradSpec *s) {
    if (m->abi_version != EDEN_GPU_ABI_VERSION)
        return g->fail(EDEN_GPU_E_INVALID, "ABI version %d, library is %d", m->abi_version, EDEN_GPU_ABI_VERSION);
    if (!finite_pos(m->dt)) return g->fail(EDEN_GPU_E_INVALID, "dt must be positive");
    if (m->n_izh != 0 || m->n_pois != 0 || m->n_wave != 0 || m->n_clamp != 0 || m->n_gap != 0 || m->n_graded != 0)
        return g->fail(EDEN_GPU_E_INVALID,
                       "gradients cover independent physical cells with HH channels, pulse inputs and synaptic drive "
                       "with fixed events: the model has %d point neurons, %lld Poisson, %lld waveform and %lld clamp "
                       "inputs and %lld gap-junction and graded-synapse ends",
                       m->n_izh, (long long)m->n_pois, (long long)m->n_wave, (long long)m->n_clamp,
                       (long long)(m->n_gap + m->n_graded));
    if (m->cable_solver != EDEN_CABLE_BWD_EULER)
        return g->fail(EDEN_GPU_E_INVALID, "gradients follow the backward-Euler cable solve only");
    for (int k = 0; k < m->n_syn_types; k++) {
        const EdenGpuSynapseType &t = m->syn_types[k];
        if ((t.kind != EDEN_SYN_EXPONE && t.kind != EDEN_SYN_EXPTWO) || !std::isfinite(t.gbase) ||
            !std::isfinite(t.erev) || !finite_pos(t.tau_decay) || (t.kind == EDEN_SYN_EXPTWO && !finite_pos(t.tau_rise)))
            return g->fail(EDEN_GPU_E_INVALID, "synapse type %d: bad parameters", k);
    }
    for (int64_t k = 0; k < m->n_syn; k++) {
        const int src = m->syn_src[k];
        if (src < 0 || src >= m->n_src) return g->fail(EDEN_GPU_E_INVALID, "synapse %lld: bad source", (long long)k);
        if (m->src_target[src] >= 0)
            return g->fail(EDEN_GPU_E_INVALID,
                           "synapse %lld: its presynaptic cell %d spikes, so its events depend on the parameters; "
                           "gradients need synaptic events fixed in advance (spike sources without a membrane)",
                           (long long)k, src);
        if (m->syn_target[k] < 0 || m->syn_target[k] >= m->n_comp || m->syn_type[k] < 0 ||
            m->syn_type[k] >= m->n_syn_types || !(m->syn_delay[k] >= 0.0f) || !std::isfinite(m->syn_delay[k]) ||
            !std::isfinite(m->syn_weight[k]))
            return g->fail(EDEN_GPU_E_INVALID, "synapse %lld: bad target, type, delay or weight", (long long)k);
    }
    for (int64_t k = 0; k < m->n_timed; k++) {
        if (m->timed_target[k] < 0 || m->timed_target[k] >= m->n_comp || m->timed_type[k] < 0 ||
            m->timed_type[k] >= m->n_syn_types || !std::isfinite(m->timed_weight[k]) ||
            m->timed_off[k + 1] < m->timed_off[k])
            return g->fail(EDEN_GPU_E_INVALID, "timed input %lld: bad target, type, weight or steps", (long long)k);
    }
    for (int64_t e = 0; e < m->n_ext; e++)
        if (m->ext_src[e] < 0 || m->ext_src[e] >= m->n_src || (e > 0 && m->ext_step[e] < m->ext_step[e - 1]))
            return g->fail(EDEN_GPU_E_INVALID, "spike-source events must name a source and be sorted by step");
    if (m->n_phys <= 0 || m->n_comp <= 0) return g->fail(EDEN_GPU_E_INVALID, "no physical cells");
    for (int k = 0; k < m->n_chan_types; k++)
        for (int q = 0; q < m->chan_types[k].n_gates && q < EDEN_MAX_GATES; q++)
            if (m->chan_types[k].gate_kind[q] != EDEN_GATE_RATES)
                return g->fail(EDEN_GPU_E_INVALID,
                               "gradients cover gateHHrates gates: channel type %d gate %d is of another kind", k, q);
    if (m->phys_comp_off[0] != 0 || m->phys_comp_off[m->n_phys] != m->n_comp)
        return g->fail(EDEN_GPU_E_INVALID, "phys_comp_off must span [0, n_comp]");
    for (int c = 0; c < m->n_phys; c++) {
        const int a = m->phys_comp_off[c], b = m->phys_comp_off[c + 1];
        if (b <= a) return g->fail(EDEN_GPU_E_INVALID, "cell %d has no compartments", c);
        if (m->comp_parent[a] != -1) return g->fail(EDEN_GPU_E_INVALID, "cell %d: compartment 0 must be the root", c);
        for (int i = a + 1; i < b; i++) {
            const int p = m->comp_parent[i];
            if (p < 0 || p >= i - a)
                return g->fail(EDEN_GPU_E_INVALID, "cell %d compartment %d: parent %d must precede it", c, i - a, p);
            if (!finite_pos(m->comp_r_axial[i])) return g->fail(EDEN_GPU_E_INVALID, "compartment %d: bad axial resistance", i);
        }
    }
    for (int i = 0; i < m->n_comp; i++) {
        if (!finite_pos(m->comp_c[i])) return g->fail(EDEN_GPU_E_INVALID, "compartment %d: bad capacitance", i);
        if (!std::isfinite(m->comp_area[i]) || !std::isfinite(m->comp_inv_rc[i]) || !std::isfinite(m->comp_v0[i]))
            return g->fail(EDEN_GPU_E_INVALID, "compartment %d: non-finite constant", i);
        if (m->comp_chan_off[i + 1] < m->comp_chan_off[i]) return g->fail(EDEN_GPU_E_INVALID, "comp_chan_off not monotone");
    }
    if (m->comp_chan_off[0] != 0) return g->fail(EDEN_GPU_E_INVALID, "comp_chan_off[0] != 0");
    const int n_chan = m->comp_chan_off[m->n_comp];
    for (int ch = 0; ch < n_chan; ch++)
        if (m->chan_type[ch] < 0 || m->chan_type[ch] >= m->n_chan_types)
            return g->fail(EDEN_GPU_E_INVALID, "channel %d: bad type", ch);
    for (int k = 0; k < m->n_chan_types; k++) {
        const EdenGpuChannelType &t = m->chan_types[k];
        if (t.n_gates < 0 || t.n_gates > EDEN_MAX_GATES) return g->fail(EDEN_GPU_E_INVALID, "channel type %d: gate count", k);
        for (int q = 0; q < t.n_gates; q++) {
            if (t.gate_instances[q] < 0 || t.gate_instances[q] > 16) return g->fail(EDEN_GPU_E_INVALID, "gate instances");
            if (t.fwd_kind[q] < 0 || t.fwd_kind[q] > 2 || t.rev_kind[q] < 0 || t.rev_kind[q] > 2)
                return g->fail(EDEN_GPU_E_INVALID, "channel type %d gate %d: rate kind", k, q);
        }
    }
    for (int64_t k = 0; k < m->n_pulse; k++)
        if (m->pulse_target[k] < 0 || m->pulse_target[k] >= m->n_comp)
            return g->fail(EDEN_GPU_E_INVALID, "pulse %lld: target out of range", (long long)k);
    if (s->n_params < 0) return g->fail(EDEN_GPU_E_INVALID, "negative parameter count");
    if (s->n_steps < 1) return g->fail(EDEN_GPU_E_INVALID, "n_steps must be at least 1");
    if (s->checkpoint_every < 0) return g->fail(EDEN_GPU_E_INVALID, "checkpoint_every must not be negative");
    if (s->n_rec < 0 || (s->n_rec > 0 && !s->rec_comp)) return g->fail(EDEN_GPU_E_INVALID, "recorded compartments missing");
    for (int r = 0; r < s->n_rec; r++)
        if (s->rec_comp[r] < 0 || s->rec_comp[r] >= m->n_comp)
            return g->fail(EDEN_GPU_E_INVALID, "recorded compartment %d out of range", r);
    std::vector<char> chan_use(s->n_params, 0), ra_use(s->n_params, 0);
    if (s->chan_param)
        for (int ch = 0; ch < n_chan; ch++) {
            const int p = s->chan_param[ch];
            if (p < -1 || p >= s->n_params) return g->fail(EDEN_GPU_E_INVALID, "channel %d: parameter %d out of range", ch, p);
            if (p >= 0) chan_use[p] = 1;
        }
    if (s->cell_ra_param)
        for (int c = 0; c < m->n_phys; c++) {
            const int p = s->cell_ra_param[c];
            if (p < -1 || p >= s->n_params) return g->fail(EDEN_GPU_E_INVALID, "cell %d: parameter %d out of range", c, p);
            if (p >= 0) {
                if (!s->cell_ra || !finite_pos(s->cell_ra[c]))
                    return g->fail(EDEN_GPU_E_INVALID, "cell %d: resistivity parameter without a positive cell_ra", c);
                ra_use[p] = 1;
            }
        }
    for (int p = 0; p < s->n_params; p++)
        if (chan_use[p] && ra_use[p])
            return g->fail(EDEN_GPU_E_INVALID, "parameter %d is both a conductivity and a resistivity", p);
    auto weight_params = [&](const int32_t *par, int64_t n, const char *what) {
        if (!par) return 0;
        for (int64_t k = 0; k < n; k++) {
            const int p = par[k];
            if (p < -1 || p >= s->n_params)
                return g->fail(EDEN_GPU_E_INVALID, "%s %lld: parameter %d out of range", what, (long long)k, p);
            if (p >= 0 && (chan_use[p] || ra_use[p]))
                return g->fail(EDEN_GPU_E_INVALID, "parameter %d is both a weight and a conductivity or resistivity", p);
        }
        return 0;
    };
    int rc = weight_params(s->syn_param, m->n_syn, "synapse");
    if (rc) return rc;
    return weight_params(s->timed_param, m->n_timed, "timed input");
}

// Host layout: each cell's compartments breadth-first (children in increasing
// order, so a node's children are consecutive), channels and pulses in that
// order, per-cell parameter slots and recorded columns.
int build(EdenGpuGrad *g, const EdenGpuModel *m, const EdenGpuGradSpec *s) {
    const float dt = m->dt;
    const int nphys = m->n_phys;
    GradDev &d = g->d;
    d.n_cells = nphys;
    d.n_rec = s->n_rec;
    d.S = s->checkpoint_every > 0 ? s->checkpoint_every : 100;
    d.N = s->n_steps;
    d.n_comp = m->n_comp;
    d.dt = dt;
    std::vector<int32_t> cell_c0(nphys + 1, 0), cell_g0(nphys + 1, 0), cell_ch0(nphys + 1, 0), cell_l0(nphys + 1, 0),
        cell_s0(nphys + 1, 0), cell_r0(nphys + 1, 0), cell_ra_slot(nphys, -1), cell_ra_param(nphys, -1),
        cell_chain(nphys, 0);
    std::vector<float> cell_ra(nphys, 1.0f);
    std::vector<int32_t> lev, P(m->n_comp), CB(m->n_comp), CE(m->n_comp), comp_ch0, comp_pu0;
    std::vector<float> C(m->n_comp), A(m->n_comp), IRC(m->n_comp), U(m->n_comp, 0.0f), L(m->n_comp, 0.0f),
        V0(m->n_comp);
    std::vector<int32_t> ch_type, ch_g0, ch_param, ch_slot;
    std::vector<float> ch_gbase, ch_erev, pu_start, pu_dur, pu_aw;
    std::vector<int32_t> new_of(m->n_comp);  // model compartment -> breadth-first position
    // pulses by compartment, in pulse order
    std::vector<std::vector<int64_t>> pulses_of(m->n_comp);
    for (int64_t k = 0; k < m->n_pulse; k++) pulses_of[m->pulse_target[k]].push_back(k);
    int64_t n_gate = 0;
    comp_pu0.push_back(0);
    for (int c = 0; c < nphys; c++) {
        const int a = m->phys_comp_off[c], b = m->phys_comp_off[c + 1], nc = b - a;
        std::vector<std::vector<int>> kids(nc);
        for (int i = 1; i < nc; i++) kids[m->comp_parent[a + i]].push_back(i);
        std::vector<int> order, depth_of(nc, 0);
        order.reserve(nc);
        order.push_back(0);
        std::vector<int> pos(nc, 0);
        lev.push_back(0);
        int cur_depth = 0;
        for (size_t h = 0; h < order.size(); h++) {
            const int i = order[h];
            if (depth_of[i] != cur_depth) {
                lev.push_back((int)h);
                cur_depth = depth_of[i];
            }
            pos[i] = (int)h;
            for (int k : kids[i]) {
                depth_of[k] = depth_of[i] + 1;
                order.push_back(k);
            }
        }
        lev.push_back(nc);
        cell_l0[c + 1] = (int32_t)lev.size();
        bool chain = true;  // breadth-first order of an unbranched cable from its end
        for (int h = 0; h + 1 < nc && chain; h++) chain = kids[order[h]].size() == 1 && pos[kids[order[h]][0]] == h + 1;
        cell_chain[c] = chain ? 1 : 0;
        const int gbase_cell = (int)n_gate;
        const int ch_first = (int)ch_type.size();
        std::vector<int32_t> slots;  // parameter of each local slot
        auto slot_of = [&](int p) {
            for (size_t k = 0; k < slots.size(); k++)
                if (slots[k] == p) return (int)k;
            slots.push_back(p);
            return (int)slots.size() - 1;
        };
        for (int h = 0; h < nc; h++) {
            const int i = order[h], gi = a + i, gn = a + h;
            new_of[gi] = gn;
            const int p = m->comp_parent[gi];
            P[gn] = p >= 0 ? pos[p] : -1;
            CB[gn] = kids[i].empty() ? 0 : pos[kids[i].front()];
            CE[gn] = kids[i].empty() ? 0 : pos[kids[i].front()] + (int)kids[i].size();
            C[gn] = m->comp_c[gi];
            A[gn] = m->comp_area[gi];
            IRC[gn] = m->comp_inv_rc[gi];
            V0[gn] = m->comp_v0[gi];
            if (p >= 0) {
                const float R = m->comp_r_axial[gi];
                U[gn] = -dt / (R * m->comp_c[gi]);
                L[gn] = -dt / (R * m->comp_c[a + p]);
            }
            comp_ch0.push_back((int32_t)ch_type.size() - ch_first);  // local to the cell
            for (int ch = m->comp_chan_off[gi]; ch < m->comp_chan_off[gi + 1]; ch++) {
                const int pp = s->chan_param ? s->chan_param[ch] : -1;
                ch_type.push_back(m->chan_type[ch]);
                ch_g0.push_back((int32_t)(n_gate - gbase_cell));
                ch_param.push_back(pp);
                ch_slot.push_back(pp >= 0 ? slot_of(pp) : -1);
                ch_gbase.push_back(m->chan_gbase[ch]);
                ch_erev.push_back(m->chan_erev[ch]);
                n_gate += m->chan_types[m->chan_type[ch]].n_gates;
            }
            for (int64_t k : pulses_of[gi]) {
                pu_start.push_back(m->pulse_start[k]);
                pu_dur.push_back(m->pulse_duration[k]);
                pu_aw.push_back(m->pulse_amplitude[k] * m->pulse_weight[k]);
            }
            comp_pu0.push_back((int32_t)pu_start.size());
        }
        if (s->cell_ra_param && s->cell_ra_param[c] >= 0) {
            cell_ra_param[c] = s->cell_ra_param[c];
            cell_ra[c] = s->cell_ra[c];
            cell_ra_slot[c] = slot_of(s->cell_ra_param[c]);
        }
        if ((int)slots.size() > kMaxSlots)
            return g->fail(EDEN_GPU_E_INVALID, "cell %d uses %d parameters, at most %d", c, (int)slots.size(), kMaxSlots);
        for (int32_t p : slots) g->slot_param.push_back(p);
        cell_c0[c + 1] = b;
        cell_g0[c + 1] = (int32_t)n_gate;
        cell_ch0[c + 1] = (int32_t)ch_type.size();
        cell_s0[c + 1] = (int32_t)g->slot_param.size();
        g->dims.c = std::max(g->dims.c, nc);
        g->dims.g = std::max(g->dims.g, (int)(n_gate - gbase_cell));
        g->dims.ch = std::max(g->dims.ch, (int)ch_type.size() - ch_first);
        g->dims.slots = std::max(g->dims.slots, (int)slots.size());
    }
    if (n_gate > INT32_MAX) return g->fail(EDEN_GPU_E_INVALID, "too many gates");
    d.n_gate = n_gate;
    // recorded columns grouped by cell
    std::vector<int32_t> cell_of(m->n_comp);
    for (int c = 0; c < nphys; c++)
        for (int i = m->phys_comp_off[c]; i < m->phys_comp_off[c + 1]; i++) cell_of[i] = c;
    std::vector<std::vector<int32_t>> rec_by_cell(nphys);
    for (int r = 0; r < s->n_rec; r++) rec_by_cell[cell_of[s->rec_comp[r]]].push_back(r);
    std::vector<int32_t> rec_local, rec_col;
    for (int c = 0; c < nphys; c++) {
        for (int32_t r : rec_by_cell[c]) {
            rec_local.push_back(new_of[s->rec_comp[r]] - cell_c0[c]);
            rec_col.push_back(r);
        }
        cell_r0[c + 1] = (int32_t)rec_local.size();
    }
    // step times: the reference accumulates the float dt in double from 0
    // at step 1 and runs each step at that time as a float
    std::vector<float> tk((size_t)d.N + 1, 0.0f);
    double time = 0.0;
    for (int64_t n = 1; n <= d.N; n++) {
        tk[n] = (float)time;
        time += (double)dt;
    }
    // ---- synaptic drive: each item's firing steps (timed inputs: listed;
    // connections from spike sources: the reference's delivery and single
    // pending-spike rule, eden/Eden.cpp:3646-3686, replayed on the source's
    // spikes), then groups of one compartment, kind and synapse type --
    // inputs before connections, types in increasing order -- with their
    // items in model order
    struct Item { int comp, kind, type, param; float w; std::vector<int32_t> ev; };
    std::vector<Item> items;
    {
        std::vector<std::vector<int64_t>> spikes_of(m->n_src);
        for (int64_t e = 0; e < m->n_ext; e++)
            if (m->ext_step[e] >= 1 && m->ext_step[e] < d.N) spikes_of[m->ext_src[e]].push_back(m->ext_step[e]);
        auto due_step = [&](float p) -> int64_t {  // step k in 1 .. N-1 with tk[k] <= p < tk[k] + dt
            const auto it = std::upper_bound(tk.begin() + 1, tk.begin() + d.N, p);
            const int64_t j = (int64_t)(it - tk.begin()) - 1;
            for (int64_t k = std::max<int64_t>(1, j - 1); k <= j && k < d.N; k++)
                if (tk[k] <= p && p < tk[k] + dt) return k;
            return 0;
        };
        for (int64_t k = 0; k < m->n_timed; k++) {
            Item it{new_of[m->timed_target[k]], 0, m->timed_type[k], s->timed_param ? s->timed_param[k] : -1,
                    m->timed_weight[k], {}};
            for (int64_t e = m->timed_off[k]; e < m->timed_off[k + 1]; e++)
                if (m->timed_step[e] >= 1 && m->timed_step[e] < d.N) it.ev.push_back((int32_t)m->timed_step[e]);
            items.push_back(std::move(it));
        }
        for (int64_t k = 0; k < m->n_syn; k++) {
            Item it{new_of[m->syn_target[k]], 1, m->syn_type[k], s->syn_param ? s->syn_param[k] : -1,
                    m->syn_weight[k], {}};
            const float delay = m->syn_delay[k];
            float pend = -INFINITY;
            for (int64_t step : spikes_of[m->syn_src[k]]) {
                const float t = tk[step], fresh = t + delay, tdt = t + dt;
                if (t <= fresh && fresh < tdt) it.ev.push_back((int32_t)step);
                if (pend < tdt && pend < fresh) {
                    pend = fresh;
                    const int64_t kd = due_step(pend);
                    if (kd > 0) it.ev.push_back((int32_t)kd);
                }
            }
            std::sort(it.ev.begin(), it.ev.end());
            it.ev.erase(std::unique(it.ev.begin(), it.ev.end()), it.ev.end());
            items.push_back(std::move(it));
        }
        std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) {
            if (a.comp != b.comp) return a.comp < b.comp;
            if (a.kind != b.kind) return a.kind < b.kind;
            return a.type < b.type;
        });
    }
    std::vector<int32_t> comp_gr0(m->n_comp + 1, 0), gr_kind, gr_it0, it_grp, it_type, it_param, it_ev;
    std::vector<int64_t> it_ev0{0};
    std::vector<float> gr_erev, it_w;
    for (size_t i = 0; i < items.size(); i++) {
        const Item &it = items[i];
        if (i == 0 || it.comp != items[i - 1].comp || it.kind != items[i - 1].kind || it.type != items[i - 1].type) {
            gr_kind.push_back(it.kind);
            gr_erev.push_back(m->syn_types[it.type].erev);
            gr_it0.push_back((int32_t)i);
            comp_gr0[it.comp + 1]++;
        }
        it_grp.push_back((int32_t)gr_kind.size() - 1);
        it_type.push_back(it.type);
        it_param.push_back(it.param);
        it_w.push_back(it.w);
        it_ev.insert(it_ev.end(), it.ev.begin(), it.ev.end());
        it_ev0.push_back((int64_t)it_ev.size());
    }
    gr_it0.push_back((int32_t)items.size());
    for (int i = 0; i < m->n_comp; i++) comp_gr0[i + 1] += comp_gr0[i];
    std::vector<GradSyn> syn(std::max(m->n_syn_types, 1));
    for (int k = 0; k < m->n_syn_types; k++) {
        const EdenGpuSynapseType &t = m->syn_types[k];
        syn[k] = GradSyn{t.kind, t.gbase, t.tau_decay, t.tau_rise, t.weight_prop * t.waveform_factor};
    }
    d.n_grp = (int32_t)gr_kind.size();
    d.n_item = (int64_t)items.size();
    g->item_param = it_param;
    g->cell_ra_param = cell_ra_param;
    // shared memory per warp
    const Dims &dm = g->dims;
    d.n_types = m->n_chan_types;
    g->smem = (size_t)dm.slots * 32 * sizeof(double) + (size_t)m->n_chan_types * sizeof(EdenGpuChannelType) +
              (size_t)(10 * dm.c + 2 * dm.g + 2 * dm.ch) * sizeof(float) +
              (size_t)(4 * dm.c + 1 + 3 * dm.ch) * sizeof(int32_t);
    int optin = 0;
    GTRY(g, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, g->device));
    if (g->smem > (size_t)optin)
        return g->fail(EDEN_GPU_E_INVALID, "largest cell (%d compartments, %d gates) needs %zu bytes of shared memory, "
                                           "the device allows %d", dm.c, dm.g, g->smem, optin);
    if (g->smem > 48 * 1024) {
        GTRY(g, cudaFuncSetAttribute(k_grad_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g->smem));
        GTRY(g, cudaFuncSetAttribute(k_grad_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g->smem));
    }
    std::vector<EdenGpuChannelType> types(m->chan_types, m->chan_types + m->n_chan_types);
    int rc;
#define UP(dst, src) \
    if ((rc = upload(g, &d.dst, src)) != 0) return rc
    UP(cell_c0, cell_c0); UP(cell_g0, cell_g0); UP(cell_ch0, cell_ch0); UP(cell_l0, cell_l0); UP(cell_s0, cell_s0); UP(cell_r0, cell_r0);
    UP(cell_ra_slot, cell_ra_slot); UP(cell_ra_param, cell_ra_param); UP(cell_chain, cell_chain); UP(cell_ra, cell_ra); UP(lev, lev);
    UP(C, C); UP(A, A); UP(IRC, IRC); UP(U, U); UP(L, L); UP(V0, V0);
    UP(P, P); UP(CB, CB); UP(CE, CE); UP(comp_ch0, comp_ch0); UP(comp_pu0, comp_pu0);
    UP(ch_type, ch_type); UP(ch_g0, ch_g0); UP(ch_param, ch_param); UP(ch_slot, ch_slot);
    UP(ch_gbase, ch_gbase); UP(ch_erev, ch_erev); UP(types, types);
    UP(pu_start, pu_start); UP(pu_dur, pu_dur); UP(pu_aw, pu_aw);
    UP(rec_local, rec_local); UP(rec_col, rec_col); UP(tk, tk);
    UP(comp_gr0, comp_gr0); UP(gr_kind, gr_kind); UP(gr_it0, gr_it0); UP(it_grp, it_grp); UP(it_type, it_type);
    UP(it_param, it_param); UP(it_ev, it_ev); UP(it_ev0, it_ev0); UP(gr_erev, gr_erev); UP(it_w, it_w);
    UP(syn, syn);
#undef UP
    if (d.n_grp > 0) {
        const size_t rows = (size_t)(d.N + 1) * d.n_grp;
        if ((rc = alloc(g, &d.gtab, rows)) != 0) return rc;
        if ((rc = alloc(g, &d.gbar, rows)) != 0) return rc;
        if ((rc = alloc(g, &d.it_a, (size_t)d.n_item)) != 0) return rc;
        if ((rc = alloc(g, &d.it_b, (size_t)d.n_item)) != 0) return rc;
        if ((rc = alloc(g, &d.it_cur, (size_t)d.n_item)) != 0) return rc;
        if ((rc = alloc(g, &d.item_grad, (size_t)d.n_item)) != 0) return rc;
        GTRY(g, cudaMemset(d.gbar, 0, rows * sizeof(float)));
    }
    const int64_t n_ck = d.N >= 2 ? (d.N - 2) / d.S + 1 : 1;
    if ((rc = alloc(g, &g->d_params, (size_t)std::max(s->n_params, 1))) != 0) return rc;
    d.params = g->d_params;
    if ((rc = alloc(g, &d.ck_v, (size_t)n_ck * m->n_comp)) != 0) return rc;
    if ((rc = alloc(g, &d.ck_q, (size_t)n_ck * n_gate)) != 0) return rc;
    if ((rc = alloc(g, &d.tr_v, (size_t)(d.S + 1) * m->n_comp)) != 0) return rc;
    if ((rc = alloc(g, &d.tr_q, (size_t)(d.S + 1) * n_gate)) != 0) return rc;
    if ((rc = alloc(g, &g->d_trace, (size_t)d.N * std::max(s->n_rec, 1))) != 0) return rc;
    d.trace = g->d_trace;
    if ((rc = alloc(g, &g->d_tgrad, (size_t)d.N * std::max(s->n_rec, 1))) != 0) return rc;
    d.trace_grad = g->d_tgrad;
    if ((rc = alloc(g, &g->d_slot, g->slot_param.size())) != 0) return rc;
    d.slot_grad = g->d_slot;
    g->n_params = s->n_params;
    g->n_cells = nphys;
    g->n_rec = s->n_rec;
    return 0;
}

}  // namespace

extern "C" int edenGpuGradCreate(const EdenGpuModel *model, const EdenGpuGradSpec *spec, EdenGpuGrad **out) {
    if (!out) return EDEN_GPU_E_INVALID;
    EdenGpuGrad *g = new EdenGpuGrad();
    *out = g;
    if (!model || !spec) return g->fail(EDEN_GPU_E_INVALID, "null model or spec");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return g->fail(EDEN_GPU_E_NODEVICE, "no CUDA device visible");
    }
    g->device = spec->device;
    if (g->device < 0 || g->device >= ndev) return g->fail(EDEN_GPU_E_INVALID, "device %d not present", g->device);
    GTRY(g, cudaSetDevice(g->device));
    int rc = validate(g, model, spec);
    if (rc) return rc;
    GTRY(g, cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    GTRY(g, cudaEventCreate(&g->e0));
    GTRY(g, cudaEventCreate(&g->e1));
    rc = build(g, model, spec);
    if (rc) return rc;
    GTRY(g, cudaDeviceSynchronize());
    return 0;
}

extern "C" int edenGpuGradForward(EdenGpuGrad *g, const float *params, float *trace) {
    if (!g) return EDEN_GPU_E_INVALID;
    if (!g->stream) return g->fail(EDEN_GPU_E_INVALID, "gradient context was not created");
    if (g->n_params > 0 && !params) return g->fail(EDEN_GPU_E_INVALID, "params missing");
    GTRY(g, cudaSetDevice(g->device));
    g->h_params.assign(std::max(g->n_params, 1), 0.0f);
    if (g->n_params > 0)
        GTRY(g, cudaMemcpy(g->h_params.data(), params, sizeof(float) * g->n_params, cudaMemcpyDefault));
    for (int c = 0; c < g->n_cells; c++) {
        const int p = g->cell_ra_param[c];
        if (p >= 0 && !finite_pos(g->h_params[p]))
            return g->fail(EDEN_GPU_E_INVALID, "parameter %d (a resistivity) must be positive, is %g", p, g->h_params[p]);
    }
    for (int p = 0; p < g->n_params; p++)
        if (!std::isfinite(g->h_params[p])) return g->fail(EDEN_GPU_E_INVALID, "parameter %d is not finite", p);
    GTRY(g, cudaMemcpyAsync(g->d_params, g->h_params.data(), sizeof(float) * g->h_params.size(), cudaMemcpyHostToDevice,
                            g->stream));
    GTRY(g, cudaEventRecord(g->e0, g->stream));
    if (g->d.n_grp > 0) k_grad_drive<<<(g->d.n_grp + 127) / 128, 128, 0, g->stream>>>(g->d);
    k_grad_forward<<<g->n_cells, 32, g->smem, g->stream>>>(g->d, g->dims);
    GTRY(g, cudaGetLastError());
    GTRY(g, cudaEventRecord(g->e1, g->stream));
    if (trace && g->n_rec > 0)
        GTRY(g, cudaMemcpyAsync(trace, g->d_trace, sizeof(float) * (size_t)g->d.N * g->n_rec, cudaMemcpyDefault,
                                g->stream));
    GTRY(g, cudaStreamSynchronize(g->stream));
    float ms = 0.0f;
    GTRY(g, cudaEventElapsedTime(&ms, g->e0, g->e1));
    g->fwd_ms = ms;
    g->have_forward = true;
    return 0;
}

extern "C" int edenGpuGradBackward(EdenGpuGrad *g, const float *trace_grad, float *param_grad) {
    if (!g) return EDEN_GPU_E_INVALID;
    if (!g->have_forward) return g->fail(EDEN_GPU_E_INVALID, "edenGpuGradBackward needs an edenGpuGradForward first");
    if (!param_grad && g->n_params > 0) return g->fail(EDEN_GPU_E_INVALID, "param_grad missing");
    if (!trace_grad && g->n_rec > 0) return g->fail(EDEN_GPU_E_INVALID, "trace_grad missing");
    GTRY(g, cudaSetDevice(g->device));
    if (g->n_rec > 0)
        GTRY(g, cudaMemcpyAsync(g->d_tgrad, trace_grad, sizeof(float) * (size_t)g->d.N * g->n_rec, cudaMemcpyDefault,
                                g->stream));
    GTRY(g, cudaEventRecord(g->e0, g->stream));
    k_grad_backward<<<g->n_cells, 32, g->smem, g->stream>>>(g->d, g->dims);
    if (g->d.n_item > 0) k_grad_weights<<<(unsigned)((g->d.n_item + 127) / 128), 128, 0, g->stream>>>(g->d);
    GTRY(g, cudaGetLastError());
    GTRY(g, cudaEventRecord(g->e1, g->stream));
    std::vector<double> slots(g->slot_param.size()), items((size_t)g->d.n_item);
    if (!slots.empty())
        GTRY(g, cudaMemcpyAsync(slots.data(), g->d_slot, sizeof(double) * slots.size(), cudaMemcpyDeviceToHost, g->stream));
    if (!items.empty())
        GTRY(g, cudaMemcpyAsync(items.data(), g->d.item_grad, sizeof(double) * items.size(), cudaMemcpyDeviceToHost,
                                g->stream));
    GTRY(g, cudaStreamSynchronize(g->stream));
    float ms = 0.0f;
    GTRY(g, cudaEventElapsedTime(&ms, g->e0, g->e1));
    g->bwd_ms = ms;
    // per parameter, the cells' terms in cell order
    std::vector<double> acc(std::max(g->n_params, 1), 0.0);
    for (size_t k = 0; k < slots.size(); k++) acc[g->slot_param[k]] += slots[k];
    for (size_t k = 0; k < items.size(); k++)  // the weights' terms in item order
        if (g->item_param[k] >= 0) acc[g->item_param[k]] += items[k];
    std::vector<float> out(std::max(g->n_params, 1));
    for (int p = 0; p < g->n_params; p++) out[p] = (float)acc[p];
    if (g->n_params > 0) GTRY(g, cudaMemcpy(param_grad, out.data(), sizeof(float) * g->n_params, cudaMemcpyDefault));
    return 0;
}

extern "C" int edenGpuGradTiming(EdenGpuGrad *g, double *forward_ms, double *backward_ms) {
    if (!g) return EDEN_GPU_E_INVALID;
    if (forward_ms) *forward_ms = g->fwd_ms;
    if (backward_ms) *backward_ms = g->bwd_ms;
    return 0;
}

extern "C" const char *edenGpuGradLastError(EdenGpuGrad *g) { return g ? g->err.c_str() : "null gradient context"; }

extern "C" void edenGpuGradDestroy(EdenGpuGrad *g) {
    if (!g) return;
    if (g->stream) {
        cudaSetDevice(g->device);
        cudaStreamSynchronize(g->stream);
    }
    for (void *p : g->allocs) cudaFree(p);
    if (g->e0) cudaEventDestroy(g->e0);
    if (g->e1) cudaEventDestroy(g->e1);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}
