// Device functions of libeden_gpu: one step of EDEN's loop, split into the
// phases of the reference's generated per-cell kernel, over structure-of-arrays
// device tables.  The kernels that drive them are in eden_gpu.cu:
//   * the per-step path launches k_inputs -> k_targets -> k_hines -> k_deliver
//     once per step (the reference runs one OpenMP pass per step);
//   * the windowed path (k_window) advances each group of cells K steps in one
//     CTA with its membrane state in shared memory, because within K <= min
//     synaptic delay / dt steps no cell can affect another; one k_deliver then
//     fans the window's spikes out.
//
// Internal layout (built on the host in eden_gpu.cu):
//   groups    contiguous cell ranges, one CTA each in k_window;
//   forests   each group's physical cells split into warp-sized "forests"; a
//             forest's compartments are numbered breadth-first over all its
//             cells at once, so each tree depth is one contiguous range and
//             every node's children are contiguous, in increasing original
//             index; a forest is solved by one warp;
//   targets   every membrane potential: forest compartments, then the group's
//             izhikevich neurons;
//   inputs    connection synapses, Poisson inputs and pulses sorted by target;
//             targets with any input are listed in `in_tgt` (one warp each).
#pragma once
#include <cstdint>

#include "eden_math.cuh"

namespace eden {

struct ChanTypeDev {
    int n_gates;
    int inst[EDEN_MAX_GATES];
    int fk[EDEN_MAX_GATES];
    float fr[EDEN_MAX_GATES], fm[EDEN_MAX_GATES], fs[EDEN_MAX_GATES];
    int rk[EDEN_MAX_GATES];
    float rr[EDEN_MAX_GATES], rm[EDEN_MAX_GATES], rs[EDEN_MAX_GATES];
    float q10[EDEN_MAX_GATES];
};
struct SynTypeDev {
    int kind;
    float gbase, erev, tau_decay, tau_rise, wf_w;  // wf_w = weight_prop * waveform_factor
};

__constant__ ChanTypeDev c_chan_types[kMaxChanTypes];
__constant__ SynTypeDev c_syn_types[kMaxSynTypes];

enum : int { ST_OK = 0, ST_LOG_OVERFLOW = 1 };

struct DevModel {
    int32_t n_target, n_src, n_group, n_forest, n_in;
    int64_t n_syn, n_pois;
    float dt;
    // targets
    float *v[2];
    float *diag;
    const float *c_cm, *c_inv_rc, *c_area, *c_u, *c_l;  // U = -dt/(R C_i), L = -dt/(R C_parent)
    const int32_t *c_nchild, *c_child0, *c_parent;   // internal target indices; parent -1 at roots
    const int32_t *t_izh;                            // izhikevich index or -1
    // forests: physical compartments [fo_t0, fo_t1), depth boundaries lvl[fo_l0 .. fo_l0 + fo_nlev]
    const int32_t *fo_t0, *fo_t1, *fo_l0, *fo_nlev, *lvl;
    // channels
    const int32_t *c_chan0, *ch_type, *ch_gate0;
    const float *ch_gbase, *ch_erev;
    float *gate;
    // izhikevich, structure of arrays
    const float *iz_C, *iz_v0, *iz_k, *iz_vr, *iz_vt, *iz_vpeak, *iz_a, *iz_b, *iz_c, *iz_d;
    float *iz_u;
    // per-target input ranges and the list of targets with inputs
    const int32_t *t_pulse0, *t_pois0;
    const int64_t *t_syn0;
    const int32_t *in_tgt;
    const float *pu_start, *pu_dur, *pu_amp, *pu_w;
    // Poisson inputs
    float *po_ts, *po_isi, *po_a, *po_b;
    const float *po_rate, *po_w;
    const int32_t *po_seed, *po_inst;
    const uint8_t *po_type;
    // connection synapses
    float *sy_a, *sy_b, *sy_pend;
    uint32_t *sy_mask;
    const float *sy_w, *sy_delay;
    const uint8_t *sy_type;
    // per-target input currents of the current step (per-step path)
    float *in_I, *in_G, *syn_I, *syn_G;
    // spike sources and fan-out (source -> synapses, connection order)
    const int32_t *t_src;
    const float *src_thr;
    const int64_t *fan0;
    const int32_t *fan_syn;
    // window spike lists (double-buffered by window parity) and the spike log
    int32_t *wspk_src[2];
    int32_t *wspk_step[2];
    int32_t *wspk_count;  // [2]
    int32_t *log_src;
    int64_t *log_step;
    unsigned long long *log_count;
    int64_t log_cap;
    // trajectory recording: CSR target -> recorded columns
    const int32_t *t_trace0, *trace_col;
    int32_t n_trace;
    float *trace_buf;
    int64_t trace_cap;
    // groups for k_window
    const int32_t *g_t0, *g_t1, *g_f0, *g_f1, *g_i0, *g_i1;
    int32_t *status;
};

// Per-window arguments: the window covers steps [step0, step0 + K); steps
// <= 0 are initialisation passes.  The previous window began at step
// step0 - Kprev at time t_prev0; its triggers are the mask bits 1..Kprev-1
// (replayed before step0) and bit Kprev (the trigger of step0 itself).
struct WindowArgs {
    int64_t step0;
    int32_t K, Kprev;
    double t0, t_prev0;
    int32_t par;   // which V buffer holds the state at step0
    int32_t wpar;  // window parity: which spike list this window fills
};

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// ---------------------------------------------------------------------------
// spike compaction: warp ballot, one atomic per warp
// ---------------------------------------------------------------------------
__device__ __forceinline__ void push_spike(const DevModel &m, bool spiked, int32_t src, int32_t log_step,
                                           int wpar) {
    unsigned active = __activemask();
    unsigned ballot = __ballot_sync(active, spiked);
    if (ballot == 0) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&m.wspk_count[wpar], __popc(ballot));
    base = __shfl_sync(active, base, leader);
    if (spiked) {
        int rank = __popc(ballot & ((1u << lane) - 1));
        m.wspk_src[wpar][base + rank] = src;
        m.wspk_step[wpar][base + rank] = log_step;
    }
}

// ---------------------------------------------------------------------------
// synapses and inputs
// ---------------------------------------------------------------------------
// State update + exposure of expOne (native, eden/Eden.cpp:3424-3466) or
// expTwo (LEMS forward Euler; OnEvent replaces the decay on that step).
__device__ __forceinline__ void synapse_dyn(const SynTypeDev &st, bool init, float dt, bool fire, float v,
                                            float w, float &a, float &b, float &iw, float &gw) {
    if (st.kind == EDEN_SYN_EXPONE) {
        float g = a;
        float i = g * (st.erev - v);
        if (!init) {
            float an = a - dt * (a / st.tau_decay);
            if (fire) an = a + st.gbase;
            a = an;
        }
        iw = i * w;
        gw = g * w;
    } else {
        float g = st.gbase * (b - a);
        float i = g * (st.erev - v);
        if (init) {
            a = 0.0f;
            b = 0.0f;
        } else {
            float an = a + dt * (-a / st.tau_rise);
            float bn = b + dt * (-b / st.tau_decay);
            if (fire) {
                an = a + st.wf_w;
                bn = b + st.wf_w;
            }
            a = an;
            b = bn;
        }
        iw = i * w;
        gw = g * w;
    }
}

// Pending-spike rule for a trigger read at time t (eden/Eden.cpp:3646-3686):
// fire now if t <= t+delay < t+dt; keep it as the single pending spike only if
// the old one is already due (pend < t+dt) and earlier than the new one.
__device__ __forceinline__ bool trigger_arrival(float t, float dt, float delay, float &pend) {
    float fresh = t + delay;
    bool now = (t <= fresh && fresh < t + dt);
    if (pend < t + dt && pend < fresh) pend = fresh;
    return now;
}

// Replay triggers of the previous window (bits 1..Kprev-1) and return the
// trigger of the window's first step (bit Kprev).  Exact because every delay
// is at least Kprev * dt, so none of these spikes can fall due before step0.
__device__ __forceinline__ bool replay_mask(uint32_t mask, const WindowArgs &w, float dt, float delay,
                                            float &pend) {
    double t = w.t_prev0;
    for (int b = 1; b < w.Kprev; b++) {
        t += (double)dt;
        if ((mask >> b) & 1u) trigger_arrival((float)t, dt, delay, pend);
    }
    return (mask >> w.Kprev) & 1u;
}

// One poissonFiringSynapse for one step (LEMS_CoreComponents.inc.xml:623-672):
// the spiker fires its own synapse instance on the step its OnCondition holds.
__device__ __forceinline__ void pois_step(const DevModel &m, int64_t k, bool init, int64_t step, float v,
                                          float &iw, float &gw) {
    float ts = m.po_ts[k], isi = m.po_isi[k], a = m.po_a[k], b = m.po_b[k];
    float avg_isi = 1.0f / m.po_rate[k];
    bool fired = false;
    if (init) {
        ts = 0.0f;
        isi = (-avg_isi) * logf(1.0f - randof(1.0f, (int64_t)m.po_seed[k], m.po_inst[k], step, 0));
    } else if (ts > isi) {
        ts = 0.0f;
        isi = (-avg_isi) * logf(1.0f - randof(1.0f, (int64_t)m.po_seed[k], m.po_inst[k], step, 1));
        fired = true;
    } else {
        ts = ts + m.dt * 1.0f;
    }
    synapse_dyn(c_syn_types[m.po_type[k]], init, m.dt, fired, v, m.po_w[k], a, b, iw, gw);
    m.po_ts[k] = ts;
    m.po_isi[k] = isi;
    m.po_a[k] = a;
    m.po_b[k] = b;
}

// One connection synapse for one step; `first` = first step of a window,
// where the previous window's triggers are read (and the mask cleared).
__device__ __forceinline__ void syn_step(const DevModel &m, int64_t s, const WindowArgs &w, bool init, bool first,
                                         float t, float v, float &iw, float &gw) {
    float pend = m.sy_pend[s], a = m.sy_a[s], b = m.sy_b[s];
    bool fire = false;
    if (!init) {
        if (first) {
            uint32_t mask = m.sy_mask[s];
            if (mask) {
                m.sy_mask[s] = 0;
                float delay = m.sy_delay[s];
                bool trig = replay_mask(mask, w, m.dt, delay, pend);
                if (t <= pend && pend < t + m.dt) fire = true;
                if (trig && trigger_arrival(t, m.dt, delay, pend)) fire = true;
            } else if (t <= pend && pend < t + m.dt) {
                fire = true;
            }
        } else if (t <= pend && pend < t + m.dt) {
            fire = true;
        }
    }
    synapse_dyn(c_syn_types[m.sy_type[s]], init, m.dt, fire, v, m.sy_w[s], a, b, iw, gw);
    m.sy_pend[s] = pend;
    m.sy_a[s] = a;
    m.sy_b[s] = b;
}

// Input and synapse currents into target t, computed by a whole warp: each
// lane updates every 32nd item and the partial sums are combined by a
// butterfly reduction, so every lane returns the same totals.
// (The reference sums the same terms sequentially, eden/Eden.cpp:5927-5945.)
__device__ __forceinline__ void inputs_warp(const DevModel &m, int t, const WindowArgs &w, int64_t step, float time,
                                            bool first, float v, float &Iin, float &Gin, float &Isyn, float &Gsyn) {
    const int lane = threadIdx.x & 31;
    const bool init = step <= 0;
    float ip = 0.0f;
    const int q0 = m.t_pulse0[t], q1 = m.t_pulse0[t + 1];
    for (int q = q0 + lane; q < q1; q += 32) {
        float s = m.pu_start[q];
        if (s <= time && time <= s + m.pu_dur[q]) ip += m.pu_amp[q] * m.pu_w[q];
    }
    float pi = 0.0f, pg = 0.0f;
    const int p0 = m.t_pois0[t], p1 = m.t_pois0[t + 1];
    for (int p = p0 + lane; p < p1; p += 32) {
        float iw, gw;
        pois_step(m, p, init, step, v, iw, gw);
        pi += iw;
        pg += gw;
    }
    float si = 0.0f, sg = 0.0f;
    const int64_t s0 = m.t_syn0[t], s1 = m.t_syn0[t + 1];
    for (int64_t s = s0 + lane; s < s1; s += 32) {
        float iw, gw;
        syn_step(m, s, w, init, first, time, v, iw, gw);
        si += iw;
        sg += gw;
    }
    if (q1 > q0) ip = warp_sum(ip);
    if (p1 > p0) {
        pi = warp_sum(pi);
        pg = warp_sum(pg);
    }
    if (s1 > s0) {
        si = warp_sum(si);
        sg = warp_sum(sg);
    }
    Iin = ip + pi;
    Gin = pg;
    Isyn = si;
    Gsyn = sg;
}

// ---------------------------------------------------------------------------
// targets
// ---------------------------------------------------------------------------
// One target for one step: the trajectory sample, then either the channels +
// voltage pre-update of a compartment (eden/Eden.cpp:5013-6107), writing the
// pre-updated V to *x and the Hines diagonal to *d, or the izhikevich2007
// update (LEMS_CoreComponents.inc.xml:1140-1185), writing v' to *x.
__device__ __forceinline__ void target_step(const DevModel &m, int t, bool init, int64_t step, float v, float Iin,
                                            float Gin, float Isyn, float Gsyn, float *x, float *d, int wpar) {
    if (!init) {
        for (int k = m.t_trace0[t]; k < m.t_trace0[t + 1]; k++) {
            int64_t row = (step - 1) % m.trace_cap;
            m.trace_buf[row * m.n_trace + m.trace_col[k]] = v;
        }
    }
    int iz = m.t_izh[t];
    if (iz < 0) {
        float A = m.c_area[t];
        float Ich = 0.0f, Gch = 0.0f;
        for (int ch = m.c_chan0[t]; ch < m.c_chan0[t + 1]; ch++) {
            const ChanTypeDev &ct = c_chan_types[m.ch_type[ch]];
            float fopen = 1.0f;
            float *q = m.gate + m.ch_gate0[ch];
            for (int g = 0; g < ct.n_gates; g++) {
                float qo = q[g];
                float alpha = rate_value(ct.fk[g], ct.fr[g], ct.fm[g], ct.fs[g], v);
                float beta = rate_value(ct.rk[g], ct.rr[g], ct.rm[g], ct.rs[g], v);
                float tau = 1.0f / (alpha + beta);
                float inf = alpha / (alpha + beta);
                float qn;
                if (init) {
                    qn = inf;
                } else {
                    float blend = expf(-((m.dt * ct.q10[g]) / tau));
                    qn = blend * qo + (1.0f - blend) * inf;
                    if (!(qn > 1e-6f)) qn = 1e-6f;
                    if (!(qn < (float)(1 - 1e-6))) qn = (float)(1 - 1e-6);
                }
                q[g] = qn;
                for (int r = 0; r < ct.inst[g]; r++) fopen = fopen * qo;
            }
            float gs = m.ch_gbase[ch] * fopen;
            Ich += (gs * (m.ch_erev[ch] - v) * 1e-5f) * A;
            Gch += (gs * 1e-5f) * A;
        }
        float I = Ich + Iin + Isyn;
        float G = Gch + Gin + Gsyn;
        float C = m.c_cm[t];
        *d = 1.0f * (G / C) + m.c_inv_rc[t];
        *x = init ? v : v + (m.dt * (I + (v * G))) / C;
    } else {
        float u = m.iz_u[iz];
        float vr = m.iz_vr[iz];
        float iext = Isyn + Iin;
        float imemb = ((m.iz_k[iz] * (v - vr)) * 1e-3f) * (v - m.iz_vt[iz]) + iext - u;
        float vn, un;
        bool spike = false;
        if (init) {
            vn = m.iz_v0[iz];
            un = 0.0f;
        } else {
            vn = v + m.dt * (imemb / m.iz_C[iz]);
            float du = (m.iz_a[iz] * ((m.iz_b[iz] * (v - vr)) - u)) * 1e-3f;
            un = u + m.dt * du * 1e3f;
            if (v > m.iz_vpeak[iz]) {
                vn = m.iz_c[iz];
                un = u + m.iz_d[iz];
                spike = true;
            }
        }
        *x = vn;
        m.iz_u[iz] = un;
        int src = m.t_src[t];
        push_spike(m, spike && src >= 0, src, (int32_t)(step + 1), wpar);
    }
}

// ---------------------------------------------------------------------------
// cable solve
// ---------------------------------------------------------------------------
// Backward-Euler Hines solve of one forest by one warp (eden/Eden.cpp:6114-6225),
// on arrays indexed by (internal target - base): D (diagonal, in), X (the
// pre-updated V, solved in place), U, L (off-diagonals).  Depths are processed
// deepest first; each node pulls its children's elimination terms in
// increasing child order, the same sequence of operations as the reference's
// depth-first post-order.  Back-substitution then runs root-first.  Ends with
// the threshold test V < thr < V_next of the forest's spike sources
// (eden/Eden.cpp:6247-6252).
__device__ __forceinline__ void hines_forest(const DevModel &m, int f, bool init, int64_t step, float *D, float *X,
                                             const float *U, const float *L, const float *Vin, int base,
                                             int wpar) {
    const int lane = threadIdx.x & 31;
    const int c0 = m.fo_t0[f], c1 = m.fo_t1[f];
    if (!init && c1 > c0) {
        const float dt = m.dt;
        for (int c = c0 + lane; c < c1; c += 32) D[c - base] = 1.0f + D[c - base] * dt;
        __syncwarp();
        const int32_t *lv = m.lvl + m.fo_l0[f];
        const int nlev = m.fo_nlev[f];
        for (int lev = nlev - 2; lev >= 0; lev--) {
            for (int j = lv[lev] + lane; j < lv[lev + 1]; j += 32) {
                int n = m.c_nchild[j];
                if (n == 0) continue;
                int ch = m.c_child0[j] - base;
                float dj = D[j - base], xj = X[j - base];
                for (int k = 0; k < n; k++) {
                    float ratio = L[ch + k] / D[ch + k];
                    dj -= ratio * U[ch + k];
                    xj -= ratio * X[ch + k];
                }
                D[j - base] = dj;
                X[j - base] = xj;
            }
            __syncwarp();
        }
        for (int r = lv[0] + lane; r < lv[1]; r += 32) X[r - base] = X[r - base] / D[r - base];
        __syncwarp();
        for (int lev = 1; lev < nlev; lev++) {
            for (int i = lv[lev] + lane; i < lv[lev + 1]; i += 32)
                X[i - base] = (X[i - base] - U[i - base] * X[m.c_parent[i] - base]) / D[i - base];
            __syncwarp();
        }
    }
    for (int c0w = c0; c0w < c1; c0w += 32) {
        int c = c0w + lane;
        bool spk = false;
        int src = -1;
        if (c < c1) {
            src = m.t_src[c];
            if (src >= 0) {
                float thr = m.src_thr[src];
                spk = (Vin[c - base] < thr && thr < X[c - base]);
            }
        }
        push_spike(m, spk, src, (int32_t)(step + 1), wpar);
    }
}

}  // namespace eden
