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
#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

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
    int gk[EDEN_MAX_GATES];  // EDEN_GATE_*, then the timeCourse and steadyState forms
    int tk[EDEN_MAX_GATES];
    float tr[EDEN_MAX_GATES], tm[EDEN_MAX_GATES], ts[EDEN_MAX_GATES];
    int ik[EDEN_MAX_GATES];
    float ir[EDEN_MAX_GATES], im[EDEN_MAX_GATES], is[EDEN_MAX_GATES];
};
struct SynTypeDev {
    int kind;
    float gbase, erev, tau_decay, tau_rise, wf_w;  // wf_w = weight_prop * waveform_factor
    float r_decay, r_rise;                          // correctly rounded 1 / tau
    float f_decay, f_rise;                          // 1 - dt / tau, one step's decay factor
    float c_alpha;                                  // alpha kinds: e dt / tau, g' = f g + c A
    // blockingPlasticSynapse: plasticity (plastic != 0) with release
    // probability p and one step's factors 1 - dt/tau_rec, 1 - dt/tau_fac
    // (f_fac 1: U stays p)
    int plastic;
    float rel_p, f_rec, f_fac;
};

// x / tau, correctly rounded, from r = RN(1/tau): q = RN(x*r) is within an
// ulp of the quotient, the residual x - tau*q is exact in one FMA, and
// RN(q + r*residual) is the correctly rounded quotient (Markstein's
// theorem, the basis of software division on FMA machines).  The residual
// is exact only away from the underflow range, so an operand below 2^-100
// is scaled by 2^64 first (exact) and the quotient scaled back (exact unless
// the quotient itself is subnormal, where it may differ from the correctly
// rounded one by one subnormal ulp, 2^-149).  Branch-free: synapse states
// that have decayed to tiny values or zero are common, and a divergent
// branch to a hardware division there cost more than the division saves.
__device__ __forceinline__ float div_by_tau(float x, float tau, float r) {
    const bool tiny = fabsf(x) < 0x1p-100f;
    const float xs = tiny ? x * 0x1p64f : x;
    const float q = xs * r;
    const float e = fmaf(-q, tau, xs);
    const float qs = fmaf(e, r, q);
    return tiny ? qs * 0x1p-64f : qs;
}


enum : int { ST_OK = 0, ST_LOG_OVERFLOW = 1 };
enum : int { BK_PULSE = 0, BK_POIS = 1, BK_SYN = 2, BK_TIMED = 3 };
// block-level only: a voltage clamp's sum of weight / R, applied as -V g
// (its chunks run as pulse-block type kClampB)
enum : int { BK_CLAMPV = 4 };
// a synapse block of a current-based kind (alphaCurrentSynapse) carries this
// flag beside its kind: its exposure is a current, with no conductance
enum : int { BK_KIND_MASK = 7, BK_CURRENT = 8, BK_BLOCK = 16 };
// pulse-block types: 0 pulses, then the waveform shapes, then the two halves of a clamp
enum : int { kPulseSine = 1 + EDEN_WAVE_SINE, kPulseRamp = 1 + EDEN_WAVE_RAMP, kClampA = 3, kClampB = 4 };
constexpr int kMaxWindow = 31;  // trigger bits 1..K of a 32-bit mask
constexpr int kChunkItems = 128; // input items per chunk (one warp, up to four per lane)
constexpr int kPowLen = 33;      // powers 0..32 of a synapse decay factor
constexpr int kWaveWords = 8;    // waveform input record: delay, duration, 3 shape parameters, weight, 2 spare
constexpr int kClampWords = 8;   // clamp record: delay, duration, 3 phase targets, R, weight, spare

struct DevModel {
    int32_t n_target, n_src, n_group, n_forest, n_in;
    // channel and synapse type tables (per context, so that contexts of
    // different models can run side by side)
    const ChanTypeDev *chan_types;
    const SynTypeDev *syn_types;
    int64_t n_syn, n_pois;
    float dt;
    // targets
    float *v[2];
    float *diag;
    const float *c_cm, *c_inv_rc, *c_area, *c_u, *c_l;  // U = -dt/(R C_i), L = -dt/(R C_parent)
    const int32_t *c_cend, *c_parent;  // end of each node's child range; parent (internal, -1 at roots)
    const int32_t *t_izh;                            // izhikevich index or -1
    // forward-Euler cable update (fwd_euler != 0): each node's axial
    // resistance to its parent and the start of its child range
    int32_t fwd_euler;
    const float *c_rax;
    const int32_t *c_kb;
    // windowed-path constants of each physical compartment.  A "flat"
    // compartment has one gateless channel, no inputs, is no spike source and
    // has only flat compartments below it; everything else is "non-flat".
    //   c_kl   flat: the pre-update increment dt*(G*E)/C (V' = V + c_kl, the
    //          reference's V + dt*(I + V*G)/C with I = G*(E - V)); non-flat:
    //          its L (its elimination factor is L / pivot, rebuilt each step)
    //   c_pv0  flat: reciprocal of its Hines pivot, which is the same every
    //          step because nothing below it changes; non-flat: unused
    //   c_rt0  flat: L / pivot, its elimination factor into its parent
    //   c_cep  child-range end | child-range begin << 10 | (parent + 1) << 20
    //          | non-flat << 30, all local to the compartment's forest
    const float *c_kl, *c_pv0, *c_rt0;
    const uint32_t *c_cep;
    // forests: physical compartments [fo_t0, fo_t1), depth boundaries lvl[fo_l0 .. fo_l0 + fo_nlev]
    const int32_t *fo_t0, *fo_t1, *fo_l0, *fo_nlev, *lvl;
    // channels
    const int32_t *c_chan0, *ch_type, *ch_gate0;
    const float *ch_gbase, *ch_erev;
    float *gate;
    // point neurons: kind, parameters field-major ([EDEN_POINT_PARAMS][n_izh]),
    // two state variables besides V (izhikevich u, adEx w; last spike time)
    int32_t n_izh;
    const int32_t *iz_kind;
    const float *iz_p;
    float *iz_u, *iz_s;
    // input blocks: each target's pulses, then Poisson inputs and connection
    // synapses in runs of one synapse type; a block's conductance (or, for
    // pulses, current) for step k of the window is G[k * n_block + block]
    int32_t n_block;
    const int32_t *t_blk0;            // [n_target + 1]
    const int32_t *bk_kind;           // BK_PULSE, BK_POIS, BK_SYN, BK_TIMED
    const uint8_t *bk_type;           // synapse type of a Poisson / synapse block
    const float *bk_erev;
    const int32_t *in_tgt;            // targets with any block
    // blocks are cut into chunks of at most kChunkItems items, one warp each; step k's
    // partial sum of chunk c is Gp[k * n_chunk + c] and a block's value is the
    // sum of its chunks' partials in chunk order
    int32_t n_chunk;
    const int32_t *bk_c0;             // [n_block + 1] chunk range of each block
    const int32_t *ck_blk;            // block of each chunk
    const int32_t *ck_info;           // kind | synapse type << 2 | items << 8
    const int64_t *ck_i0;             // first item of each chunk
    const int32_t *ck_n;              // items in the chunk
    float *Gp;                        // [32 * n_chunk]
    const float *syn_pow;             // per synapse type: f_rise^j, then f_decay^j, j < kPowLen
    int32_t pois_exact;               // dt is a whole number of us: Poisson clocks advance exactly
    float *ck_a, *ck_b;               // aggregate synapse state of each chunk (weighted sums)
    const float *pu_start, *pu_dur, *pu_amp, *pu_w;
    const float *gate_ext;            // per channel type and gate, kGateExtWords (gate_next_p)
    const float *wv_p;                // sine / ramp generators, kWaveWords per item
    const float *cl_p;                // voltage clamps, kClampWords per item
    // Poisson inputs
    float *po_ts, *po_isi, *po_a, *po_b;  // po_a/po_b: own synapse state just after its last event
    int32_t *po_last;                      // step of that event
    const float *po_rate, *po_w;
    const int32_t *po_seed, *po_inst;
    const int32_t *po_rng;                 // random-call id of the input's first draw
    const uint8_t *po_type;
    // timedSynapticInput items: own synapse state (as Poisson items), weight,
    // type, the steps each fires in (tm_step[tm_off[i] .. tm_off[i+1]]) and
    // the next one due
    float *tm_a, *tm_b;
    int32_t *tm_last;
    const float *tm_w;
    const uint8_t *tm_type;
    const int64_t *tm_off, *tm_step;
    int64_t *tm_cur;
    // connection synapses
    float *sy_a, *sy_b, *sy_pend;     // sy_a/sy_b: state just after the synapse's last event
    float *sy_R, *sy_U;               // blockingPlasticSynapse: plasticity state after the last event
    const float2 *bk_block;           // per input block: the voltage block's ratio and scaling voltage
    int32_t *sy_last;                 // step of that event
    uint32_t *sy_mask;
    const float *sy_w, *sy_delay;
    const uint8_t *sy_type;
    // spike sources and fan-out (source -> synapses, connection order)
    const int32_t *t_src;
    const float *src_thr;
    const int64_t *fan0;
    const int32_t *fan_syn;
    // spikes of the sources with no target, in step order: source, logging step
    const int32_t *ext_src, *ext_step;
    // window spike lists (double-buffered by window parity) and the spike log;
    // *_time: the threshold-crossing time (us) interpolated in double
    // between the step's starting and final potential (NaN where there is
    // none: point neurons and sources with no membrane)
    int32_t *wspk_src[2];
    int32_t *wspk_step[2];
    double *wspk_time[2];
    int32_t *wspk_count;  // [2]
    int32_t *log_src;
    int64_t *log_step;
    double *log_time;
    unsigned long long *log_count;
    int64_t log_cap;
    // trajectory recording: CSR target -> recorded columns
    const int32_t *t_trace0, *trace_col;
    const int32_t *trace_gate;  // per listed column: the gate slot it records, or -1 for V
    int32_t n_trace;
    float *trace_buf;
    int64_t trace_cap;
    // units of the windowed kernel, one warp each: targets [un_t0, un_t1),
    // forest un_f (-1: a batch of izhikevich neurons), shared-memory slice at
    // word un_off of its CTA, gates [un_gt0, un_gt0 + un_ngt), spike sources
    // gs_*[un_s0 .. un_s1) and recorded targets gr_*[un_r0 .. un_r1)
    // (target indices local to the unit); CTA c runs units [cta_u0[c], cta_u0[c+1])
    int32_t n_unit;
    const int32_t *un_t0, *un_t1, *un_f, *un_off, *un_gt0, *un_ngt, *un_s0, *un_s1, *un_r0, *un_r1;
    const int32_t *cta_u0;
    // per unit: spike sources (gs_*) and trace columns [un_r0, un_r1): gr_t is
    // the unit-local target, or -1 - the unit-local gate slot of a gate's
    // state; gr_col the column
    const int32_t *gs_t, *gs_src, *gr_t, *gr_col;
    const float *gs_thr;
    // non-flat compartments of forest units: nf_t[un_nf0[u] .. un_nf1[u]) are
    // unit-local indices; spike sources (gs_t) and gates refer to these slots
    const int32_t *un_nf0, *un_nf1, *nf_t;
    // per forest depth (parallel to lvl): 0x80 if it holds a non-flat compartment
    const uint8_t *lvl_info;
    // channels of the non-flat compartments, per non-flat compartment
    // [nf_c0, nf_c1): conductivity, reversal potential, first gate (index in
    // the unit's gates) and gate count | instances << (3 + 5 * gate)
    const int32_t *nf_c0, *nf_c1;
    const int32_t *nf_sig;            // channel set of each non-flat compartment (generated code), -1: none
    const float *nfc_g, *nfc_e;
    const int32_t *nfc_q, *nfc_i;
    // per channel type and gate, the 9-word gate parameter record (gate_next_p)
    const float *gate_par;
    int32_t *status;
    // forests whose cells may lose diagonal dominance: their elimination runs
    // in double precision (hines_window_f64, hines_forest_f64); c_d0 is a
    // flat compartment's constant diagonal term G/C + sum 1/(R C); dscr is
    // the per-step path's double scratch (two per target)
    const uint8_t *fo_f64;
    const float *c_d0;
    double *dscr;
    // gap-junction ends of each target [t_gap0[t], t_gap0[t+1]): the peer
    // (internal target), conductance (uS) and weight
    const int32_t *t_gap0, *gap_peer;
    const float *gap_g, *gap_w;
    // gradedSynapse ends of each target [t_gr0[t], t_gr0[t+1]): the peer,
    // EDEN_GRADED_PARAMS parameters, weight and state s
    const int32_t *t_gr0, *gr_peer;
    const float *gr_par, *gr_w;
    float *gr_s;
};

// The gap-junction current into target t at potential v, its peers read
// from the step's starting potentials vnow: each end contributes
// (g (V_peer - v)) w, as the reference sums a synapse's exposure times its
// weight (eden/Eden.cpp:3407-3422, 3708-3710); no conductance term.
__device__ __forceinline__ float gap_current(const DevModel &m, int t, float v, const float *vnow, bool init) {
    float i = 0.0f;
    for (int k = m.t_gap0[t]; k < m.t_gap0[t + 1]; k++) i += (m.gap_g[k] * (vnow[m.gap_peer[k]] - v)) * m.gap_w[k];
    // gradedSynapse ends (LEMS_CoreComponents.inc.xml:38-80, as the
    // reference's LEMS code steps it: the derived values and the current
    // from the step's starting state, s by forward Euler, the OnCondition
    // overriding; s = 0 in the initialisation steps).  Each end's state is
    // read and written by its own target's thread, once per step.
    for (int k = m.t_gr0[t]; k < m.t_gr0[t + 1]; k++) {
        const float *p = m.gr_par + (size_t)EDEN_GRADED_PARAMS * k;  // conductance, delta, k, Vth, erev
        const float s = m.gr_s[k];
        const float inf = 1.0f / (1.0f + expf((p[3] - vnow[m.gr_peer[k]]) / p[1]));
        const float tau = (1.0f - inf) / p[2];
        i += ((p[0] * s) * (p[4] - v)) * m.gr_w[k];
        float sn = 0.0f;
        if (!init) {
            sn = s + m.dt * ((1.0f - inf) > 1e-4f ? (inf - s) / tau : 0.0f);
            if ((1.0f - inf) < 1e-4f) sn = inf;
        }
        m.gr_s[k] = sn;
    }
    return i;
}

constexpr uint32_t kCepMask = 0x3ffu;
constexpr int kCepBeginShift = 10;
constexpr int kCepParentShift = 20;
constexpr uint32_t kCepNonFlat = 1u << 30;
constexpr int kGateWords = 9;  // gate parameter record (gate_next_p)
constexpr int kGateExtWords = 9;  // a non-rates gate's kind and timeCourse / steadyState forms

// Shared-memory words of a unit's slice in the windowed kernel (an even
// count, so that every slice starts 8-byte aligned).  A forest: 6 per
// compartment in three pairs (V and elimination factor; c_kl and the packed
// child range/parent/flag; U and pivot), 10 per non-flat compartment (local index, V at
// the step start, area, C, sum of 1/(R C), input-block range, channel
// range, channel set), 4 per channel of a non-flat compartment, 11 per gate (value,
// non-flat slot, parameter record), the depth boundaries, 3 per spike
// source, 3 per input block (kind, reversal potential, chunk start) plus
// one, and the window's conductance series of the unit's input chunks
// (kcap steps).  A batch of izhikevich neurons: V
// twice and 11 parameter / state words per neuron.
__host__ __device__ inline int forest_words(int n, int nf, int nfch, int ngt, int nlev, int ns, int nblk, int nck,
                                            int kcap, bool f64 = false) {
    // a double-precision forest adds its eliminated values, pivots and
    // factors in double (6 words per compartment, 8-byte aligned)
    const int w = 6 * n + 10 * nf + 4 * nfch + (2 + kGateWords) * ngt + (nlev + 1) + 3 * ns + 3 * nblk + 1 + kcap * nck +
                  (f64 ? 6 * n + 2 : 0);
    return (w + 1) & ~1;
}
__host__ __device__ inline int izh_words(int n) { return ((2 + EDEN_POINT_PARAMS + 3) * n + 1 + 1) & ~1; }

// Per-window arguments: the window covers steps [step0, step0 + K); steps
// <= 0 are initialisation passes.  The previous window began at step
// step0 - Kprev; its triggers are the mask bits 1..Kprev-1 (replayed before
// step0) and bit Kprev (the trigger of step0 itself).
struct WindowArgs {
    double t0;     // simulation time of step0 (us), accumulated in double on the host
    int64_t step0;
    int32_t K, Kprev;
    int32_t par;   // which V buffer holds the state at step0
    int32_t wpar;  // window parity: which spike list this window fills
    int32_t ext0, ext1;  // the spikes of sources with no target logged in steps step0+1 .. step0+K
};

// Single-precision times (us) of the window's steps and of the previous
// window's, accumulated on the host in double from 0 as the reference
// accumulates its time (eden/Eden.cpp:11486, 11931).
struct WindowTimes {
    float tk[32];
    float tprev[32];
};

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// ---------------------------------------------------------------------------
// spike compaction: warp ballot, one atomic per warp
// ---------------------------------------------------------------------------
// NaN: a spike with no interpolated crossing time
__device__ __forceinline__ double no_time() { return __longlong_as_double(0x7ff8000000000000ll); }

// Staging copies: one 4-byte word from global to shared memory without a
// register round trip (cp.async), so that all of a lane's staging loads are
// in flight together; stage_wait() waits for the lane's copies, and a
// __syncwarp() after it publishes them to the warp.
__device__ __forceinline__ void stage_word(void *smem_dst, const void *gmem_src) {
    unsigned s;
    asm("{\n .reg .u64 a;\n cvta.to.shared.u64 a, %1;\n cvt.u32.u64 %0, a;\n}" : "=r"(s) : "l"(smem_dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void push_spike(const DevModel &m, bool spiked, int32_t src, int32_t log_step,
                                           int wpar, double tcross) {
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
        m.wspk_time[wpar][base + rank] = tcross;
    }
}

// The time (us) at which V crossed thr during a step that starts at time t
// (double) with potential v0 and ends with v1 (v0 < thr < v1), by linear
// interpolation in double.  A diagnostic beside the logged step: the
// reference quantises spike times to the step (eden/Eden.cpp:6247-6252).
__device__ __forceinline__ double crossing_time(double t, float dt, float v0, float v1, float thr) {
    return t + (double)dt * (((double)thr - (double)v0) / ((double)v1 - (double)v0));
}

// ---------------------------------------------------------------------------
// synapses and inputs
// ---------------------------------------------------------------------------
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
__device__ __forceinline__ bool replay_mask(uint32_t mask, const WindowArgs &w, const float *tprev, float dt,
                                            float delay, float &pend) {
    for (int b = 1; b < w.Kprev; b++)
        if ((mask >> b) & 1u) trigger_arrival(tprev[b], dt, delay, pend);
    return (mask >> w.Kprev) & 1u;
}

// ---------------------------------------------------------------------------
// input chunks: event-driven synapses with an aggregate state per chunk
// ---------------------------------------------------------------------------
// expOne and expTwo synapses are linear between events, so the weighted sum
// of a chunk's synapse states obeys the same update as one synapse (expOne
// G' = G - dt*G/tau, eden/Eden.cpp:3424-3466; expTwo A' = A - dt*A/tau_rise,
// B' = B - dt*B/tau_decay, LEMS_CoreComponents.inc.xml:145-180) and the
// chunk's conductance is its exposure (G, or gbase*(B - A)).  A synapse only
// costs work when it fires.  On that step the reference replaces the
// synapse's decay by the jump (G += gbase; A, B += weight_prop*wf), so the
// aggregate gets back the decay it applied to that synapse plus the jump,
// both times its weight.  For that the synapse keeps its own state as of its
// last event and the step of that event.

// A synapse's own state at the start of step s from its value just after its
// event at step `last`: the reference's per-step a - dt*(a/tau), in closed
// form a * f^n with f = 1 - dt/tau (used only for the decay its event replaces).
__device__ __forceinline__ float decayed(float a, float f, const float *fpow, int n) {
    if (n <= 0) return a;
    return a * (n < kPowLen ? fpow[n] : powf(f, (float)n));
}

// The contribution (dA, dB) of one synapse's event at step s to its chunk's
// aggregate, and the synapse's own state after it.
template <int KIND>
__device__ __forceinline__ void input_event(const SynTypeDev &st, const float *pw, float dt, float w, int64_t s,
                                            float &a, float &b, int32_t &last, float &dA, float &dB, float js = 1.0f) {
    const int n = (int)(s - (int64_t)last) - 1;
    if (KIND == EDEN_SYN_EXPTWO) {
        // (js: a blockingPlasticSynapse's plasticity factor for this event)
        const float jump = st.wf_w * js;
        const float ai = decayed(a, st.f_rise, pw, n), bi = decayed(b, st.f_decay, pw + kPowLen, n);
        dA = w * (dt * div_by_tau(ai, st.tau_rise, st.r_rise) + jump);
        dB = w * (dt * div_by_tau(bi, st.tau_decay, st.r_decay) + jump);
        a = ai + jump;
        b = bi + jump;
    } else {
        const float gi = decayed(a, st.f_decay, pw + kPowLen, n);
        dA = w * (dt * div_by_tau(gi, st.tau_decay, st.r_decay) + st.gbase);
        dB = 0.0f;
        a = gi + st.gbase;
    }
    last = (int32_t)s;
}

// Adds an event at window step j to the lane's rows of the event tiles,
// clearing the rows on the lane's first event of the window.
__device__ __forceinline__ void put_event(float *rowA, float *rowB, bool &used, int K, int j, float dA, float dB) {
    if (!used) {
        for (int q = 0; q < K; q++) { rowA[q] = 0.0f; rowB[q] = 0.0f; }
        used = true;
    }
    rowA[j] += dA;
    rowB[j] += dB;
}

// Poisson input `it` over the K steps of a window (poissonFiringSynapse,
// LEMS_CoreComponents.inc.xml:623-672): initialisation draws the first
// interval at each init step; afterwards the input fires its own synapse on
// the step its time since the last spike exceeds the interval (then restarts
// that time at 0 and draws the next interval), else adds dt to it.  When dt
// is a whole number of us and the times stay below 2^24 us, every such sum
// is exact, so the firing step is found directly instead of step by step.
__device__ __forceinline__ float pois_draw(const DevModel &m, int64_t it, int64_t step, int invocation) {
    return (-(1.0f / m.po_rate[it])) *
           logf(1.0f - randof(1.0f, (int64_t)m.po_seed[it], m.po_inst[it], step, m.po_rng[it] + invocation));
}

template <int KIND>
__device__ __forceinline__ void pois_fire(const DevModel &m, int64_t it, const SynTypeDev &st, int64_t s, int j, int K,
                                          float *rowA, float *rowB, bool &used) {
    float a = m.po_a[it], b = KIND == EDEN_SYN_EXPTWO ? m.po_b[it] : 0.0f;
    int32_t last = m.po_last[it];
    float dA, dB;
    input_event<KIND>(st, m.syn_pow + (size_t)m.po_type[it] * 2 * kPowLen, m.dt, m.po_w[it], s, a, b, last, dA, dB);
    m.po_a[it] = a;
    if (KIND == EDEN_SYN_EXPTWO) m.po_b[it] = b;
    m.po_last[it] = last;
    put_event(rowA, rowB, used, K, j, dA, dB);
}

template <int KIND>
__device__ __forceinline__ void pois_window(const DevModel &m, int64_t it, const WindowArgs &w, const SynTypeDev &st,
                                            float ts, float isi, float *rowA, float *rowB, bool &used) {
    const float dt = m.dt;
    if (w.step0 <= 0) {
        for (int j = 0; j < w.K; j++) {
            ts = 0.0f;
            isi = pois_draw(m, it, w.step0 + j, 0);
        }
    } else if (m.pois_exact && isi < 0x1p23f) {
        // (exact sums: no firing in the window when even its last step's
        // time since the spike stays within the interval)
        if (ts + (float)(w.K - 1) * dt <= isi) {
            m.po_ts[it] = ts + (float)w.K * dt;
            return;
        }
        int j = 0;
        while (true) {
            // first step from j on whose time since the last spike exceeds isi
            int jn = 0;
            if (!(ts > isi)) {
                jn = (int)floorf((isi - ts) / dt) + 1;
                while (jn > 1 && ts + (float)(jn - 1) * dt > isi) jn--;
                while (!(ts + (float)jn * dt > isi)) jn++;
            }
            if (j + jn >= w.K) {
                ts = ts + (float)(w.K - j) * dt;
                break;
            }
            j += jn;
            isi = pois_draw(m, it, w.step0 + j, 1);
            pois_fire<KIND>(m, it, st, w.step0 + j, j, w.K, rowA, rowB, used);
            ts = 0.0f;
            j += 1;
            if (j >= w.K) break;
        }
    } else {
        for (int j = 0; j < w.K; j++) {
            if (ts > isi) {
                ts = 0.0f;
                isi = pois_draw(m, it, w.step0 + j, 1);
                pois_fire<KIND>(m, it, st, w.step0 + j, j, w.K, rowA, rowB, used);
            } else {
                ts = ts + dt * 1.0f;
            }
        }
    }
    m.po_ts[it] = ts;
    m.po_isi[it] = isi;
}

// Connection synapse `it` over the window: replay the previous window's
// triggers (replay_mask), then fire the single pending spike on the step
// whose interval holds it (eden/Eden.cpp:3646-3686).  That step is in this
// window for at most one pending spike: a trigger replaces the pending
// spike only once it is due, and a spike read at the first step lands at
// least K steps later.  The first step's trigger fires at once only for a
// delay below dt.
template <int KIND>
__device__ __forceinline__ void syn_window(const DevModel &m, int64_t it, const WindowArgs &w, const SynTypeDev &st,
                                           const float *tk, float pend, uint32_t mask, float *rowA, float *rowB,
                                           bool &used) {
    if (w.step0 <= 0) return;  // no spikes reach a synapse during initialisation
    const float dt = m.dt;
    const float pend0 = pend;
    bool trig = false;
    float delay = 0.0f;
    if (mask) {
        m.sy_mask[it] = 0;
        delay = m.sy_delay[it];
        trig = replay_mask(mask, w, tk + 32, dt, delay, pend);
    }
    int jf = -1;
    if (pend >= tk[0] && pend < tk[w.K - 1] + dt)
        for (int j = 0; j < w.K; j++)
            if (tk[j] <= pend && pend < tk[j] + dt) { jf = j; break; }
    bool now = false;
    if (trig) now = trigger_arrival(tk[0], dt, delay, pend);
    if (pend != pend0) m.sy_pend[it] = pend;
    if (jf < 0 && !now) return;
    float a = m.sy_a[it], b = KIND == EDEN_SYN_EXPTWO ? m.sy_b[it] : 0.0f;
    int32_t last = m.sy_last[it];
    const float wt = m.sy_w[it];
    float dA, dB;
    const float *pw = m.syn_pow + (size_t)m.sy_type[it] * 2 * kPowLen;
    // a blockingPlasticSynapse's Tsodyks-Markram state (LEMS_CoreComponents.inc.xml:
    // 263-312): forward Euler from the last event, 1 - R and U - p shrinking
    // by their factor each step; the event's jump scaled by R U before the
    // event, which then sets R = R (1 - U), U = U + p (1 - U)
    const bool plastic = KIND == EDEN_SYN_EXPTWO && st.plastic;
    float R = plastic ? m.sy_R[it] : 1.0f, U = plastic ? m.sy_U[it] : 1.0f;
    auto factor = [&](int64_t s) {
        if (!plastic) return 1.0f;
        const float n = (float)(s - (int64_t)last - 1);
        R = 1.0f - (1.0f - R) * powf(st.f_rec, n);
        U = st.rel_p + (U - st.rel_p) * powf(st.f_fac, n);
        const float f = R * U;
        R = R * (1.0f - U);
        U = U + st.rel_p * (1.0f - U);
        if (st.f_fac == 1.0f) U = st.rel_p;
        return f;
    };
    if (now && jf != 0) {
        const float js = factor(w.step0);
        input_event<KIND>(st, pw, dt, wt, w.step0, a, b, last, dA, dB, js);
        put_event(rowA, rowB, used, w.K, 0, dA, dB);
    }
    if (jf >= 0) {
        const float js = factor(w.step0 + jf);
        input_event<KIND>(st, pw, dt, wt, w.step0 + jf, a, b, last, dA, dB, js);
        put_event(rowA, rowB, used, w.K, jf, dA, dB);
    }
    m.sy_a[it] = a;
    if (KIND == EDEN_SYN_EXPTWO) m.sy_b[it] = b;
    if (plastic) { m.sy_R[it] = R; m.sy_U[it] = U; }
    m.sy_last[it] = last;
}

// Input and target kinds the kernels handle: all of them in the library's
// own build; a build generated for one model (eden_codegen.cuh) defines only
// the model's, and the compiler drops the code of the others.
#ifndef EDEN_KIND_PULSE
#define EDEN_KIND_PULSE 1
#define EDEN_KIND_GATEFORMS 1
#define EDEN_KIND_CLAMP 1
#define EDEN_KIND_SINE 1
#define EDEN_KIND_RAMP 1
#define EDEN_KIND_POIS 1
#define EDEN_KIND_TIMED 1
#define EDEN_KIND_SYN 1
#define EDEN_KIND_EXPONE 1
#define EDEN_KIND_EXPTWO 1
#define EDEN_KIND_FOREST 1
#define EDEN_KIND_IZH 1
#define EDEN_KIND_GAP 1
#define EDEN_KIND_ALPHA 1
#define EDEN_KIND_CURRENT 1
#endif

// A timedSynapticInput item over the window: its synapse fires in each
// listed step (eden/Eden.cpp:3759-3790, 3859-3871: the first step whose
// t + dt exceeds a listed time, the same step), which lowering has computed.
template <int KIND>
__device__ __forceinline__ void timed_window(const DevModel &m, int64_t it, const WindowArgs &w, const SynTypeDev &st,
                                             float *rowA, float *rowB, bool &used) {
    int64_t c = m.tm_cur[it];
    const int64_t c1 = m.tm_off[it + 1];
    const int64_t end = w.step0 + w.K;
    if (c >= c1 || m.tm_step[c] >= end) return;
    float a = m.tm_a[it], b = KIND == EDEN_SYN_EXPTWO ? m.tm_b[it] : 0.0f;
    int32_t last = m.tm_last[it];
    const float *pw = m.syn_pow + (size_t)m.tm_type[it] * 2 * kPowLen;
    for (; c < c1 && m.tm_step[c] < end; c++) {
        const int64_t s = m.tm_step[c];
        if (s < w.step0) continue;
        float dA, dB;
        input_event<KIND>(st, pw, m.dt, m.tm_w[it], s, a, b, last, dA, dB);
        put_event(rowA, rowB, used, w.K, (int)(s - w.step0), dA, dB);
    }
    m.tm_a[it] = a;
    if (KIND == EDEN_SYN_EXPTWO) m.tm_b[it] = b;
    m.tm_last[it] = last;
    m.tm_cur[it] = c;
}

// Per-warp accumulation tiles: row `lane` (stride kAccStride, padded so that
// both a row write and a column read are free of bank conflicts) holds the
// lane's terms for each step of the window.
constexpr int kAccStride = 33;

// An alpha chunk's aggregate over the window (alphaSynapse: conductance g
// and rise state A; alphaCurrentSynapse: current I and J).  Per step the
// reference integrates A' = -A / tau and g' = (e A - g) / tau by forward
// Euler (LEMS_CoreComponents.inc.xml:85-142), so over the chunk's weighted
// sums A_{j+1} = f A_j + E_j and g_{j+1} = f g_j + c A_j, f = 1 - dt / tau,
// c = e dt / tau, E_j the events of step j (each a synapse's skipped decay
// plus its jump, as input_event gives them for the expOne-like rise state).
// In closed form g_j = f^j g_0 + c j f^(j-1) A_0 + c T_j with S_j the
// events' part of A_j (a scan over the lanes, as for the other kinds) and
// T_j = sum_{k<j} f^(j-1-k) S_k a second scan over S.  Lane j keeps the
// exposure g_j of step j for Gp.
__device__ __forceinline__ void alpha_chunk_window(const DevModel &m, int c, int type, const SynTypeDev &st,
                                                   const WindowArgs &w, unsigned rows, float A, float B,
                                                   const float *tileA) {
    const int lane = threadIdx.x & 31;
    const float *pd = m.syn_pow + (size_t)type * 2 * kPowLen + kPowLen;
    const float cc = st.c_alpha;
    const float jf = (float)lane;
    // the parts from the window's starting state
    float gj = lane < w.K ? B * pd[lane] + (lane > 0 ? cc * (jf * pd[lane - 1]) * A : 0.0f) : 0.0f;
    float Ak = A * pd[w.K], Bk = B * pd[w.K] + cc * ((float)w.K * pd[w.K - 1]) * A;
    if (rows != 0) {
        float ea = 0.0f;  // lane j: the chunk's events of step j
        if (lane < w.K)
            for (unsigned r = rows; r; r &= r - 1) ea += tileA[(__ffs(r) - 1) * kAccStride + lane];
        // S: inclusive scan of the events with factor f, then exclusive
        float va = lane < w.K ? ea : 0.0f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float u = __shfl_up_sync(0xffffffffu, va, d);
            if (lane >= d) va = fmaf(pd[d], u, va);
        }
        float sj = __shfl_up_sync(0xffffffffu, va, 1);
        if (lane == 0) sj = 0.0f;
        // T: the same scan over S
        float vt = lane < w.K ? sj : 0.0f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float u = __shfl_up_sync(0xffffffffu, vt, d);
            if (lane >= d) vt = fmaf(pd[d], u, vt);
        }
        float tj = __shfl_up_sync(0xffffffffu, vt, 1);
        if (lane == 0) tj = 0.0f;
        if (lane < w.K) gj += cc * tj;
        Ak += __shfl_sync(0xffffffffu, va, w.K - 1);
        Bk += cc * __shfl_sync(0xffffffffu, vt, w.K - 1);
    }
    if (lane < w.K) m.Gp[(size_t)lane * m.n_chunk + c] = gj;
    if (lane == 0 && w.step0 > 0) { m.ck_a[c] = Ak; m.ck_b[c] = Bk; }
    __syncwarp();
}

// One chunk (at most kChunkItems items of one input block) over the K steps
// of a window, lane l handling items l, l + 32, ...  Pulses add their
// current to row l of tile A, and lane j sums column j in row order into
// Gp[j][chunk].  Synapses and Poisson inputs add their events to the tiles;
// lane j sums step j's events over the rows in row order, and every lane then
// steps the chunk's aggregate state through the window, lane j keeping the
// exposure of step j (the conductance before the step's update, as the
// reference exposes it) for Gp[j][chunk].
__device__ __forceinline__ void chunk_window(const DevModel &m, int c, int32_t info, int64_t ck_i0,
                                             const WindowArgs &w, float *tileA, float *tileB, const float *tk) {
    const int lane = threadIdx.x & 31;
    const int kind = info & 3;
    const int n = info >> 8;
    float *rowA = tileA + lane * kAccStride, *rowB = tileB + lane * kAccStride;
    if (EDEN_KIND_CLAMP && kind == BK_PULSE && ((info >> 2) & 63) >= kClampA) {
        // voltage clamps (LEMS_CoreComponents.inc.xml:555-620): the target
        // of the phase each step's time is in (the last OnCondition that
        // holds assigns); half A sums weight * target / R, half B weight / R,
        // and the cell kernel takes A - V B at the step's starting V
        const bool half_a = ((info >> 2) & 63) == kClampA;
        for (int r = 0; lane + 32 * r < n; r++) {
            const float *p = m.cl_p + (size_t)(ck_i0 + lane + 32 * r) * kClampWords;
            const float del = p[0], dur = p[1], vb = p[2], vd = p[3], va = p[4], res = p[5], wt = p[6];
            for (int j = 0; j < w.K; j++) {
                const float tf = tk[j];
                const float tv = (tf > dur + del) ? va : (tf < del) ? vb : vd;
                const bool on = w.step0 + j > 0 && tv == tv;
                const float term = on ? __fmul_rn(half_a ? tv / res : 1.0f / res, wt) : 0.0f;
                rowA[j] = r > 0 ? rowA[j] + term : term;
            }
        }
        __syncwarp();
        if (lane < w.K) {
            const int rows = n < 32 ? n : 32;
            float tot = 0.0f;
            for (int r = 0; r < rows; r++) tot += tileA[r * kAccStride + lane];
            m.Gp[(size_t)lane * m.n_chunk + c] = tot;
        }
        __syncwarp();
        return;
    }
    if ((EDEN_KIND_SINE || EDEN_KIND_RAMP) && kind == BK_PULSE && ((info >> 2) & 63) != 0) {
        // sineGenerator / rampGenerator (LEMS_CoreComponents.inc.xml:430-458,
        // 489-521): the value the OnConditions assign at the step's time,
        // which the reference's LEMS code exposes in the same step; OnStart's
        // in the initialisation passes
        const bool sine = ((info >> 2) & 63) == kPulseSine;
        for (int r = 0; lane + 32 * r < n; r++) {
            const float *p = m.wv_p + (size_t)(ck_i0 + lane + 32 * r) * kWaveWords;
            const float del = p[0], dur = p[1], a = p[2], b = p[3], cc = p[4], wt = p[5];
            for (int j = 0; j < w.K; j++) {
                const float tf = tk[j];
                const bool init = w.step0 + j <= 0;
                const bool off = tf < del || !(tf < dur + del);
                float i;
                if (sine) i = (init || off) ? 0.0f : (1.0f * a) * sinf(cc + ((2.0f * 3.14159265f) * (tf - del)) / b);
                else i = init ? cc : off ? 1.0f * cc : 1.0f * (a + ((b - a) * (tf - del)) / dur);
                const float term = __fmul_rn(i, wt);
                rowA[j] = r > 0 ? rowA[j] + term : term;
            }
        }
        __syncwarp();
        if (lane < w.K) {
            const int rows = n < 32 ? n : 32;
            float tot = 0.0f;
            for (int r = 0; r < rows; r++) tot += tileA[r * kAccStride + lane];
            m.Gp[(size_t)lane * m.n_chunk + c] = tot;
        }
        __syncwarp();
        return;
    }
    if (EDEN_KIND_PULSE && kind == BK_PULSE) {
        for (int r = 0; lane + 32 * r < n; r++) {
            const int64_t it = ck_i0 + lane + 32 * r;
            const float st = m.pu_start[it], du = m.pu_dur[it], aw = m.pu_amp[it] * m.pu_w[it];
            for (int j = 0; j < w.K; j++) {
                const float tf = tk[j];
                const float term = (st <= tf && tf <= st + du) ? aw : 0.0f;
                rowA[j] = r > 0 ? rowA[j] + term : term;
            }
        }
        __syncwarp();
        if (lane < w.K) {
            const int rows = n < 32 ? n : 32;
            float tot = 0.0f;
            for (int r = 0; r < rows; r++) tot += tileA[r * kAccStride + lane];
            m.Gp[(size_t)lane * m.n_chunk + c] = tot;
        }
        __syncwarp();
        return;
    }
    const int type = (info >> 2) & 63;
    const SynTypeDev st = m.syn_types[type];
    const bool two = st.kind == EDEN_SYN_EXPTWO || st.kind == EDEN_SYN_BLOCKING_PLASTIC;
    bool used = false;
    // the chunk's aggregate and its items' per-window state, loaded up front
    // so the loads overlap
    float A = m.ck_a[c], B = m.ck_b[c];
    const int64_t i0 = ck_i0 + lane;
    float s0v[kChunkItems / 32], s1v[kChunkItems / 32];
#pragma unroll
    for (int r = 0; r < kChunkItems / 32; r++) {
        s0v[r] = 0.0f; s1v[r] = 0.0f;
        if (lane + 32 * r < n) {
            const int64_t it = i0 + 32 * r;
            if (kind == BK_POIS) { s0v[r] = m.po_ts[it]; s1v[r] = m.po_isi[it]; }
            else if (kind == BK_SYN) { s0v[r] = m.sy_pend[it]; s1v[r] = __uint_as_float(m.sy_mask[it]); }
        }
    }
#pragma unroll
    for (int r = 0; r < kChunkItems / 32; r++) {
        if (lane + 32 * r < n) {
            const int64_t it = i0 + 32 * r;
            // only the input kinds the kernels are compiled for (all, or the model's)
            if (kind == BK_TIMED) {
                if (EDEN_KIND_TIMED) {
                    if (two) { if (EDEN_KIND_EXPTWO) timed_window<EDEN_SYN_EXPTWO>(m, it, w, st, rowA, rowB, used); }
                    else if (EDEN_KIND_EXPONE) timed_window<EDEN_SYN_EXPONE>(m, it, w, st, rowA, rowB, used);
                }
            } else if (kind == BK_POIS) {
                if (EDEN_KIND_POIS) {
                    if (two) { if (EDEN_KIND_EXPTWO) pois_window<EDEN_SYN_EXPTWO>(m, it, w, st, s0v[r], s1v[r], rowA, rowB, used); }
                    else if (EDEN_KIND_EXPONE) pois_window<EDEN_SYN_EXPONE>(m, it, w, st, s0v[r], s1v[r], rowA, rowB, used);
                }
            } else if (EDEN_KIND_SYN) {
                const uint32_t mask = __float_as_uint(s1v[r]);
                if (two) { if (EDEN_KIND_EXPTWO) syn_window<EDEN_SYN_EXPTWO>(m, it, w, st, tk, s0v[r], mask, rowA, rowB, used); }
                else if (EDEN_KIND_EXPONE) syn_window<EDEN_SYN_EXPONE>(m, it, w, st, tk, s0v[r], mask, rowA, rowB, used);
            }
        }
    }
    const unsigned rows = __ballot_sync(0xffffffffu, used);
    __syncwarp();
    float gj = 0.0f;
    if (EDEN_KIND_ALPHA && (st.kind == EDEN_SYN_ALPHA || st.kind == EDEN_SYN_ALPHA_CURRENT)) {
        alpha_chunk_window(m, c, type, st, w, rows, A, B, tileA);
        return;
    }
    if (rows == 0) {
        // no event in the window: the aggregate decays in closed form,
        // A f^j, from the factors' powers (syn_pow)
        const float *pr = m.syn_pow + (size_t)type * 2 * kPowLen, *pd = pr + kPowLen;
        if (lane < w.K) gj = two ? st.gbase * (B * pd[lane] - A * pr[lane]) : A * pd[lane];
        if (w.step0 > 0) {
            A = A * (two ? pr[w.K] : pd[w.K]);
            B = two ? B * pd[w.K] : B;
        }
        if (lane < w.K) m.Gp[(size_t)lane * m.n_chunk + c] = gj;
        if (lane == 0) { m.ck_a[c] = A; m.ck_b[c] = B; }
        __syncwarp();
        return;
    }
    float ea = 0.0f, eb = 0.0f;  // lane j: the chunk's events of step j
    if (lane < w.K)
        for (unsigned r = rows; r; r &= r - 1) {
            const int q = __ffs(r) - 1;
            ea += tileA[q * kAccStride + lane];
            eb += tileB[q * kAccStride + lane];
        }
    // the aggregate over the window: with one step's decay factor f,
    // X_j = f^j X_0 + sum_{i<j} f^(j-1-i) e_i, the sums by a scan over the lanes
    const float *pr = m.syn_pow + (size_t)type * 2 * kPowLen, *pd = pr + kPowLen;
    const float *pa = two ? pr : pd;
    float va = lane < w.K ? ea : 0.0f, vb = lane < w.K ? eb : 0.0f;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float ua = __shfl_up_sync(0xffffffffu, va, d), ub = __shfl_up_sync(0xffffffffu, vb, d);
        if (lane >= d) {
            va = fmaf(pa[d], ua, va);
            vb = fmaf(pd[d], ub, vb);
        }
    }
    // lane j: sums of the events before step j
    float sa = __shfl_up_sync(0xffffffffu, va, 1), sb = __shfl_up_sync(0xffffffffu, vb, 1);
    if (lane == 0) { sa = 0.0f; sb = 0.0f; }
    if (lane < w.K) {
        const float Aj = A * pa[lane] + sa, Bj = B * pd[lane] + sb;
        gj = two ? st.gbase * (Bj - Aj) : Aj;
    }
    const float ta = __shfl_sync(0xffffffffu, va, w.K - 1), tb = __shfl_sync(0xffffffffu, vb, w.K - 1);
    A = A * pa[w.K] + ta;
    B = two ? B * pd[w.K] + tb : B;
    if (lane < w.K) m.Gp[(size_t)lane * m.n_chunk + c] = gj;
    if (lane == 0) { m.ck_a[c] = A; m.ck_b[c] = B; }
    __syncwarp();
}

// Currents into target t at step j of the window from its input blocks:
// pulses add current; conductance blocks add g*(erev - v) and g, inputs
// first, then synapses, as eden/Eden.cpp:6057-6060 orders them.  BK_K and
// BK_E are the blocks' kinds and reversal potentials, BC0 their chunk ranges
// (indexed from blk0 and chk0, which may point into shared memory).
__device__ __forceinline__ void block_currents(const float *Gpk, int b0, int b1, const int32_t *BK_K,
                                               const float *BK_E, const int32_t *BC0, int chk0, float v, float &Iin,
                                               float &Gin, float &Isyn, float &Gsyn,
                                               const float2 *BK_B = nullptr) {
    Iin = 0.0f; Gin = 0.0f; Isyn = 0.0f; Gsyn = 0.0f;
    for (int bk = b0; bk < b1; bk++) {
        float g = 0.0f;
        for (int c = BC0[bk]; c < BC0[bk + 1]; c++) g += Gpk[c + chk0];
        // a blockingPlasticSynapse's voltage block (voltageConcDepBlockMechanism,
        // LEMS_CoreComponents.inc.xml:231-245) scales its conductance, so both
        // the current and the conductance term (per-step kernels only)
        if (BK_B && (BK_K[bk] & BK_BLOCK)) g = (1.0f / (1.0f + BK_B[bk].x * expf(-1.0f * (v / BK_B[bk].y)))) * g;
        const int kind = BK_K[bk] & BK_KIND_MASK;
        const bool current = EDEN_KIND_CURRENT && (BK_K[bk] & BK_CURRENT);
        if (kind == BK_PULSE) {
            Iin += g;
        } else if (EDEN_KIND_CLAMP && kind == BK_CLAMPV) {
            Iin -= v * g;
        } else if (kind == BK_POIS || kind == BK_TIMED) {
            if (current) {
                Iin += g;
            } else {
                Iin += g * (BK_E[bk] - v);
                Gin += g;
            }
        } else if (current) {
            Isyn += g;
        } else {
            Isyn += g * (BK_E[bk] - v);
            Gsyn += g;
        }
    }
}

__device__ __forceinline__ float gate_next(const ChanTypeDev &ct, int gi, bool init, float dt, float v, float qo) {
    if (EDEN_KIND_GATEFORMS && ct.gk[gi] != EDEN_GATE_RATES)
        return gate_general(ct.gk[gi], ct.fk[gi], ct.fr[gi], ct.fm[gi], ct.fs[gi], ct.rk[gi], ct.rr[gi], ct.rm[gi],
                            ct.rs[gi], ct.tk[gi], ct.tr[gi], ct.tm[gi], ct.ts[gi], ct.ik[gi], ct.ir[gi], ct.im[gi],
                            ct.is[gi], ct.q10[gi], init, dt, v, qo);
    const float alpha = rate_value(ct.fk[gi], ct.fr[gi], ct.fm[gi], ct.fs[gi], v);
    const float beta = rate_value(ct.rk[gi], ct.rr[gi], ct.rm[gi], ct.rs[gi], v);
    return gate_relax(alpha, beta, ct.q10[gi], init, dt, qo);
}

// The same from a gate's 9-word parameter record (forward form, rate,
// midpoint, scale; reverse form, rate, midpoint, scale; q10 factor), kept
// in shared memory by the windowed kernel.  A gate of another kind than
// gateHHrates carries 1 + its row of `ext` (kind, timeCourse form and its
// three values, steadyState form and its three values) in the bits of the
// first word above the forward form.
// An instantaneous gate keeps the steady state at the compartment's
// potential after the step (`vnew`), which is what the next step's currents
// read as its value.
__device__ __forceinline__ float gate_next_p(const float *P, const float *ext, bool init, float dt, float v,
                                             float vnew, float qo) {
    const int w0 = __float_as_int(P[0]);
    if (EDEN_KIND_GATEFORMS && (w0 >> 8) != 0) {
        const float *X = ext + (size_t)((w0 >> 8) - 1) * kGateExtWords;
        const int gk = __float_as_int(X[0]);
        return gate_general(gk, w0 & 0xff, P[1], P[2], P[3], __float_as_int(P[4]), P[5], P[6], P[7],
                            __float_as_int(X[1]), X[2], X[3], X[4], __float_as_int(X[5]), X[6], X[7], X[8], P[8],
                            init, dt, gk == EDEN_GATE_INSTANTANEOUS ? vnew : v, qo);
    }
    const float alpha = rate_value(w0, P[1], P[2], P[3], v);
    const float beta = rate_value(__float_as_int(P[4]), P[5], P[6], P[7], v);
    return gate_relax(alpha, beta, P[8], init, dt, qo);
}

// ---------------------------------------------------------------------------
// point neurons
// ---------------------------------------------------------------------------
// One step of a point neuron from its now state (V v, states u and s) with
// external current iext (synaptic then input currents), following the LEMS
// semantics the reference generates code from (eden/Eden.cpp:2832-2994):
// every state is integrated by forward Euler from the now state, then, where
// an OnCondition holds on the now state, its assignments (from now values)
// override; the initialisation passes apply OnStart.  Parameters are read as
// p[f * ps].  Returns whether the neuron spiked.
__device__ __forceinline__ bool point_update(int kind, const float *p, int ps, bool init, float t, float dt,
                                             float v, float iext, float &u, float &s, float &vn) {
#define PP(f) p[(f) * ps]
    bool spike = false;
    switch (kind) {
    case EDEN_POINT_IAF_TAU:
    case EDEN_POINT_IAF_TAU_REF: {
        // iafTauCell / iafTauRefCell: v' = (leakReversal - v) / tau, no synaptic input
        const bool ref = kind == EDEN_POINT_IAF_TAU_REF;
        if (init) {
            vn = PP(0);
            if (ref) s = t - PP(4);
            break;
        }
        const bool active = !ref || t > s + PP(4);
        const float rate = active ? (PP(0) - v) / PP(1) : 0.0f;
        vn = v + dt * rate;
        if (v > PP(2) && active) {
            if (ref) s = t;
            vn = PP(3);
            spike = true;
        }
        break;
    }
    case EDEN_POINT_IAF:
    case EDEN_POINT_IAF_REF: {
        // iafCell / iafRefCell: iMemb = leakConductance (leakReversal - v) + iSyn, v' = iMemb / C
        const bool ref = kind == EDEN_POINT_IAF_REF;
        if (init) {
            vn = PP(2);
            if (ref) s = t - PP(5);
            break;
        }
        const float imemb = PP(1) * (PP(2) - v) + iext;
        const bool active = !ref || t > s + PP(5);
        const float rate = active ? imemb / PP(0) : 0.0f;
        vn = v + dt * rate;
        if (v > PP(3) && active) {
            if (ref) s = t;
            vn = PP(4);
            spike = true;
        }
        break;
    }
    case EDEN_POINT_FN: {
        // fitzHughNagumoCell: V' = ((V - V^3 / 3) - W + I) / s, W' = 0.08 (V + 0.7 - 0.8 W) / s
        const float SEC = 1.0e6f;
        if (init) {
            vn = v;
            break;
        }
        const float w = u;
        vn = v + dt * ((((v - powf(v, 3.0f) / 3.0f) - w) + PP(0)) / SEC);
        u = w + dt * ((0.08f * ((v + 0.7f) - 0.8f * w)) / SEC);
        break;
    }
    case EDEN_POINT_IZH_DL: {
        // izhikevichCell: v' = (0.04 v^2 / mV + 5 v + (140 - U + I) mV) / ms,
        // U' = a (b v / mV - U) / ms; above thresh v = c mV, U += d
        const float MV = 1.0f, MS = 1000.0f;
        if (init) {
            vn = PP(0);
            u = (PP(0) * PP(3)) / MV;
            break;
        }
        const float uu = u;
        const float dv = ((0.04f * ((v * v) / MV) + 5.0f * v) + ((140.0f - uu) + iext) * MV) / MS;
        const float du = (PP(2) * ((PP(3) * v) / MV - uu)) / MS;
        vn = v + dt * dv;
        u = uu + dt * du;
        if (v > PP(1)) {
            vn = PP(4) * MV;
            u = uu + PP(5);
            spike = true;
        }
        break;
    }
    case EDEN_POINT_ADEX: {
        // adExIaFCell: iMemb = -gL (v - EL) + gL delT exp((v - VT) / delT) - w + iSyn,
        // v' = iMemb / C outside the refractory period, w' = (a (v - EL) - w) / tauw
        if (init) {
            vn = PP(2);
            u = 0.0f;
            s = t - PP(8);
            break;
        }
        const float w = u;
        const float imemb = (-1.0f * PP(1)) * (v - PP(2)) + (PP(1) * PP(6)) * expf((v - PP(3)) / PP(6)) - w + iext;
        const bool active = t > s + PP(8);
        const float rate = active ? imemb / PP(0) : 0.0f;
        vn = v + dt * rate;
        u = w + dt * ((PP(9) * (v - PP(2)) - w) / PP(7));
        if (v > PP(4) && active) {
            s = t;
            vn = PP(5);
            u = w + PP(10);
            spike = true;
        }
        break;
    }
    default: {
        // izhikevich2007Cell (LEMS_CoreComponents.inc.xml:1140-1187)
        const float uu = u, vr = PP(3);
        const float imemb = ((PP(2) * (v - vr)) * 1e-3f) * (v - PP(4)) + iext - uu;
        if (init) {
            vn = PP(1);
            u = 0.0f;
        } else {
            vn = v + dt * (imemb / PP(0));
            const float du = (PP(6) * ((PP(7) * (v - vr)) - uu)) * 1e-3f;
            u = uu + dt * du * 1e3f;
            if (v > PP(5)) {
                vn = PP(8);
                u = uu + PP(9);
                spike = true;
            }
        }
    }
    }
#undef PP
    return spike;
}

// ---------------------------------------------------------------------------
// targets
// ---------------------------------------------------------------------------
// One target for one step: the trajectory sample, then either the channels +
// voltage pre-update of a compartment (eden/Eden.cpp:5013-6107), writing the
// pre-updated V to *x and the Hines diagonal to *d, or the izhikevich2007
// update (LEMS_CoreComponents.inc.xml:1140-1185), writing v' to *x.
// Axial current into compartment t for the forward-Euler cable update
// (eden/Eden.cpp:4969-4990): (V_adj - V) / R summed over the neighbours in
// ascending compartment order -- the parent, then the children, which the
// breadth-first numbering keeps in that order -- from the potentials at the
// start of the step; R is the axial resistance of the edge's child end.
__device__ __forceinline__ float axial_current(const DevModel &m, int t, float v, const float *vin) {
    float I = 0.0f;
    const int p = m.c_parent[t];
    if (p >= 0) I += (vin[p] - v) / m.c_rax[t];
    for (int k = m.c_kb[t]; k < m.c_cend[t]; k++) I += (vin[k] - v) / m.c_rax[k];
    return I;
}

__device__ __forceinline__ void target_step(const DevModel &m, int t, bool init, int64_t step, float tnow, float v,
                                            float Iin, float Gin, float Isyn, float Gsyn, float *x, float *d, int wpar,
                                            float Iax = 0.0f) {
    if (!init) {
        for (int k = m.t_trace0[t]; k < m.t_trace0[t + 1]; k++) {
            int64_t row = (step - 1) % m.trace_cap;
            const int gq = m.trace_gate[k];
            m.trace_buf[row * m.n_trace + m.trace_col[k]] = gq < 0 ? v : m.gate[gq];
        }
    }
    int iz = m.t_izh[t];
    if (iz < 0) {
        float A = m.c_area[t];
        float Ich = 0.0f, Gch = 0.0f;
        for (int ch = m.c_chan0[t]; ch < m.c_chan0[t + 1]; ch++) {
            const ChanTypeDev &ct = m.chan_types[m.ch_type[ch]];
            float fopen = 1.0f;
            float *q = m.gate + m.ch_gate0[ch];
            for (int g = 0; g < ct.n_gates; g++) {
                const float qo = q[g];
                const float qn = gate_next(ct, g, init, m.dt, v, qo);
                q[g] = qn;
                // an instantaneous gate's value is its steady state at this V
                const float qf = (EDEN_KIND_GATEFORMS && ct.gk[g] == EDEN_GATE_INSTANTANEOUS) ? qn : qo;
                for (int r = 0; r < ct.inst[g]; r++) fopen = fopen * qf;
            }
            float gs = m.ch_gbase[ch] * fopen;
            Ich += (gs * (m.ch_erev[ch] - v) * 1e-5f) * A;
            Gch += (gs * 1e-5f) * A;
        }
        float I = Ich + Iin + Isyn;
        float G = Gch + Gin + Gsyn;
        float C = m.c_cm[t];
        *d = 1.0f * (G / C) + m.c_inv_rc[t];
        // backward Euler: the pre-updated V the Hines solve starts from;
        // forward Euler: V_next (eden/Eden.cpp:6092-6094)
        *x = init ? v : m.fwd_euler ? v + (m.dt * (I + Iax)) / C : v + (m.dt * (I + (v * G))) / C;
    } else {
        float u = m.iz_u[iz], sv = m.iz_s[iz], vn;
        const bool spike = point_update(m.iz_kind[iz], m.iz_p + iz, m.n_izh, init, tnow, m.dt, v, Isyn + Iin, u, sv, vn);
        *x = vn;
        m.iz_u[iz] = u;
        m.iz_s[iz] = sv;
        int src = m.t_src[t];
        push_spike(m, spike && src >= 0, src, (int32_t)(step + 1), wpar, no_time());
    }
}

// ---------------------------------------------------------------------------
// cable solve
// ---------------------------------------------------------------------------
// Backward-Euler Hines solve of one forest by one warp (eden/Eden.cpp:6114-6225).
// Arrays may live in shared or global memory and share one index space:
// D (diagonal, in), X (the pre-updated V, solved in place), U, L
// (off-diagonals), CE (end of each node's child range), P (parent), and LV
// (the forest's depth boundaries, nlev + 1 entries); `base` maps that index
// space back to internal target ids for the spike check.  Depths are
// processed deepest first; each node pulls its children's elimination terms
// in increasing child order, the same sequence of operations as the
// reference's depth-first post-order, and keeps the reciprocal of its final
// pivot.  Back-substitution then runs root-first.  When check_spikes is set
// it ends with the threshold test V < thr < V_next of the forest's spike
// sources (eden/Eden.cpp:6247-6252).
__device__ __forceinline__ void hines_forest(const DevModel &m, bool init, int64_t step, double tstep, float *D,
                                             float *X, const float *U, const float *L, const int32_t *CE,
                                             const int32_t *P, const int32_t *LV, int nlev, const float *Vin, int base,
                                             int wpar, bool check_spikes) {
    const int lane = threadIdx.x & 31;
    const int c0 = LV[0], c1 = LV[nlev];
    if (!init && c1 > c0) {
        const float dt = m.dt;
        for (int c = c0 + lane; c < c1; c += 32) D[c] = 1.0f + D[c] * dt;
        __syncwarp();
        for (int lev = nlev - 1; lev >= 0; lev--) {
            const int j0 = LV[lev], j1 = LV[lev + 1];
            for (int j = j0 + lane; j < j1; j += 32) {
                const int kb = (j == j0) ? j1 : CE[j - 1];
                const int ke = CE[j];
                float dj = D[j];
                if (ke > kb) {
                    float xj = X[j];
                    for (int i = kb; i < ke; i++) {
                        const float ratio = L[i] * D[i];  // D[i] holds the child's reciprocal pivot
                        dj -= ratio * U[i];
                        xj -= ratio * X[i];
                    }
                    X[j] = xj;
                }
                D[j] = __fdividef(1.0f, dj);
            }
            __syncwarp();
        }
        for (int r = LV[0] + lane; r < LV[1]; r += 32) X[r] = X[r] * D[r];
        __syncwarp();
        for (int lev = 1; lev < nlev; lev++) {
            for (int i = LV[lev] + lane; i < LV[lev + 1]; i += 32) X[i] = (X[i] - U[i] * X[P[i]]) * D[i];
            __syncwarp();
        }
    }
    if (!check_spikes) return;
    for (int c0w = c0; c0w < c1; c0w += 32) {
        const int c = c0w + lane;
        bool spk = false;
        int src = -1;
        double tc = 0.0;
        if (c < c1) {
            src = m.t_src[c + base];
            if (src >= 0) {
                const float thr = m.src_thr[src];
                spk = (Vin[c] < thr && thr < X[c]);
                if (spk) tc = crossing_time(tstep, m.dt, Vin[c], X[c], thr);
            }
        }
        push_spike(m, spk, src, (int32_t)(step + 1), wpar, tc);
    }
}

// The same solve in double precision for a forest whose rows may lose
// diagonal dominance (the per-step path; D and X are global, XD and DD the
// forest's double scratch): the pre-updated V and diagonal terms stay the
// single-precision values the step computed, the elimination and the
// back-substitution carry doubles, and X receives V_next rounded once.
__device__ __forceinline__ void hines_forest_f64(const DevModel &m, bool init, int64_t step, double tstep,
                                                 const float *D, float *X, const float *U, const float *L,
                                                 const int32_t *CE, const int32_t *P, const int32_t *LV, int nlev,
                                                 const float *Vin, double *XD, double *DD, int wpar) {
    const int lane = threadIdx.x & 31;
    const int c0 = LV[0], c1 = LV[nlev];
    if (!init && c1 > c0) {
        const double dt = m.dt;
        for (int c = c0 + lane; c < c1; c += 32) {
            DD[c] = 1.0 + (double)D[c] * dt;
            XD[c] = X[c];
        }
        __syncwarp();
        for (int lev = nlev - 1; lev >= 0; lev--) {
            const int j0 = LV[lev], j1 = LV[lev + 1];
            for (int j = j0 + lane; j < j1; j += 32) {
                const int kb = (j == j0) ? j1 : CE[j - 1];
                const int ke = CE[j];
                double dj = DD[j], xj = XD[j];
                for (int i = kb; i < ke; i++) {
                    const double ratio = (double)L[i] * DD[i];  // DD[i]: the child's reciprocal pivot
                    dj -= ratio * (double)U[i];
                    xj -= ratio * XD[i];
                }
                XD[j] = xj;
                DD[j] = 1.0 / dj;
            }
            __syncwarp();
        }
        for (int r = LV[0] + lane; r < LV[1]; r += 32) XD[r] = XD[r] * DD[r];
        __syncwarp();
        for (int lev = 1; lev < nlev; lev++) {
            for (int i = LV[lev] + lane; i < LV[lev + 1]; i += 32) XD[i] = (XD[i] - (double)U[i] * XD[P[i]]) * DD[i];
            __syncwarp();
        }
        for (int c = c0 + lane; c < c1; c += 32) X[c] = (float)XD[c];
        __syncwarp();
    }
    for (int c0w = c0; c0w < c1; c0w += 32) {
        const int c = c0w + lane;
        bool spk = false;
        int src = -1;
        double tc = 0.0;
        if (c < c1) {
            src = m.t_src[c];
            if (src >= 0) {
                const float thr = m.src_thr[src];
                spk = (Vin[c] < thr && thr < X[c]);
                if (spk) tc = crossing_time(tstep, m.dt, Vin[c], X[c], thr);
            }
        }
        push_spike(m, spk, src, (int32_t)(step + 1), wpar, tc);
    }
}

// Backward-Euler Hines solve of one forest by one warp for the windowed path,
// on the unit's shared-memory slice (eden/Eden.cpp:6114-6225), whose
// compartment terms sit in pairs so that one load brings two: XR (V, the
// elimination factor), KL (c_kl, the packed child range / parent / non-flat
// flag) and UP (U, the pivot).  Flat compartments keep the reciprocal pivot
// and the elimination factor L / pivot computed once, because their
// diagonals never change, and their pre-update (V += c_kl) is folded into
// the elimination; a non-flat compartment's pivot is rebuilt every step
// from its diagonal (UP.y holds G/C + sum 1/(RC) on entry, XR.x its
// pre-updated V) and its children's factors, in increasing child order as
// the reference's post-order visits them, and its factor from its L
// (KL.x).  The forest's levels (LV: each level's first compartment and
// whether it holds a non-flat one) put every compartment below its parent;
// the elimination runs from the last level to the roots of level 0, a
// level's compartments over the lanes, then the back-substitution runs
// root-first.  XR.x holds V_next on return.
constexpr int32_t kLvMask = 0xffff;
constexpr int32_t kLvNonFlat = 1 << 16;
__device__ __forceinline__ void hines_window(float dt, float2 *XR, const uint2 *KL, float2 *UP, const int32_t *LV,
                                             int nlev) {
    const int lane = threadIdx.x & 31;
    int end = LV[nlev] & kLvMask;
    for (int lev = nlev - 1; lev >= 0; lev--) {
        const int32_t lw = LV[lev];
        // a level wider than the warp takes two or more passes
        for (int j = (lw & kLvMask) + lane; j < end; j += 32) {
            const uint2 kl = KL[j];
            const uint32_t cep = kl.y;
            const int ke = (int)(cep & kCepMask), kb = (int)((cep >> kCepBeginShift) & kCepMask);
            if ((lw & kLvNonFlat) && (cep & kCepNonFlat)) {
                float xj = XR[j].x + 0.0f;
                float dj = 1.0f + UP[j].y * dt;
                for (int i = kb; i < ke; i++) {
                    const float2 c = XR[i];
                    dj -= c.y * UP[i].x;
                    xj -= c.y * c.x;
                }
                const float inv = __fdividef(1.0f, dj);
                UP[j].y = inv;
                XR[j] = make_float2(xj, __uint_as_float(kl.x) * inv);
            } else {
                float xj = XR[j].x + __uint_as_float(kl.x);
                // most compartments have at most two children: take those
                // without a loop, in order
                int i = kb;
                if (i < ke) { const float2 c = XR[i]; xj -= c.y * c.x; }
                if (i + 1 < ke) { const float2 c = XR[i + 1]; xj -= c.y * c.x; }
                for (i = kb + 2; i < ke; i++) { const float2 c = XR[i]; xj -= c.y * c.x; }
                XR[j].x = xj;
            }
        }
        end = lw & kLvMask;
        __syncwarp();
    }
    for (int r = (LV[0] & kLvMask) + lane; r < (LV[1] & kLvMask); r += 32) XR[r].x = XR[r].x * UP[r].y;
    __syncwarp();
    for (int lev = 1; lev < nlev; lev++) {
        const int i1 = LV[lev + 1] & kLvMask;
        for (int i = (LV[lev] & kLvMask) + lane; i < i1; i += 32) {
            const int p = (int)((KL[i].y >> kCepParentShift) & kCepMask) - 1;
            const float2 up = UP[i];
            XR[i].x = (XR[i].x - up.x * XR[p].x) * up.y;
        }
        __syncwarp();
    }
}

// hines_window in double precision, for a forest whose rows may lose
// diagonal dominance: every compartment's pivot is rebuilt each step from
// its diagonal term (UP.y: G/C + sum 1/(RC), the flat ones' constant one staged
// from c_d0), and the elimination and back-substitution carry doubles in
// XD / PVD / RTD; XR.x receives V_next rounded once.  A flat compartment's
// pre-update is its c_kl, and every compartment's L comes from Lg (global,
// indexed like the forest).  The operations are hines_window's, in its order.
__device__ __forceinline__ void hines_window_f64(float dt, float2 *XR, const uint2 *KL, const float2 *UP,
                                                 const float *Lg, const int32_t *LV, int nlev, double *XD,
                                                 double *PVD, double *RTD) {
    const int lane = threadIdx.x & 31;
    const double dtd = dt;
    int end = LV[nlev] & kLvMask;
    for (int lev = nlev - 1; lev >= 0; lev--) {
        const int32_t lw = LV[lev];
        for (int j = (lw & kLvMask) + lane; j < end; j += 32) {
            const uint2 kl = KL[j];
            const uint32_t cep = kl.y;
            const int ke = (int)(cep & kCepMask), kb = (int)((cep >> kCepBeginShift) & kCepMask);
            const float kc = (cep & kCepNonFlat) ? 0.0f : __uint_as_float(kl.x);
            double xj = (double)XR[j].x + (double)kc;
            double dj = 1.0 + (double)UP[j].y * dtd;
            for (int i = kb; i < ke; i++) {
                const double r = RTD[i];
                dj -= r * (double)UP[i].x;
                xj -= r * XD[i];
            }
            const double inv = 1.0 / dj;
            PVD[j] = inv;
            RTD[j] = (double)Lg[j] * inv;
            XD[j] = xj;
        }
        end = lw & kLvMask;
        __syncwarp();
    }
    for (int r = (LV[0] & kLvMask) + lane; r < (LV[1] & kLvMask); r += 32) XD[r] = XD[r] * PVD[r];
    __syncwarp();
    for (int lev = 1; lev < nlev; lev++) {
        const int i1 = LV[lev + 1] & kLvMask;
        for (int i = (LV[lev] & kLvMask) + lane; i < i1; i += 32) {
            const int p = (int)((KL[i].y >> kCepParentShift) & kCepMask) - 1;
            XD[i] = (XD[i] - (double)UP[i].x * XD[p]) * PVD[i];
        }
        __syncwarp();
    }
    const int n = LV[nlev] & kLvMask;
    for (int i = lane; i < n; i += 32) XR[i].x = (float)XD[i];
    __syncwarp();
}

}  // namespace eden
