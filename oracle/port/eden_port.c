/*
 * eden_port.c — CPU restatement of EDEN's per-timestep simulation loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU path is checked
 * against and the CPU baseline `bench.py` times beside it; the product never
 * links or calls it.  It runs on the same lowered model (include/eden_gpu.h)
 * the GPU library takes, and restates, in plain C with IEEE single precision,
 * what the reference's generated per-cell kernels compute:
 *
 *   step loop, 4 init passes, now/next swap   eden/Eden.cpp:11488-11938
 *   HH gates (exp-Euler, clamp) + currents    eden/Eden.cpp:5126-5259, 5678-5717, 5805-5898
 *   gate kinds (tau/inf forms), q10           eden/Eden.cpp:5223-5246, 5290-5375
 *   voltage pre-update                        eden/Eden.cpp:6057-6107
 *   Hines backward-Euler tree solve           eden/Eden.cpp:6114-6225 (order 4416-4473)
 *   synapse trigger + single pending spike    eden/Eden.cpp:3646-3686
 *   expOneSynapse                             eden/Eden.cpp:3424-3466
 *   expTwoSynapse (LEMS, forward Euler)       LEMS_CoreComponents.inc.xml:145-180, eden/Eden.cpp:2832-2994
 *   poissonFiringSynapse + randof hash RNG    LEMS_CoreComponents.inc.xml:623-672, eden/Eden.cpp:3199-3233, 3873-3912
 *   random-call numbering per compartment     eden/Eden.cpp:2450-2458, 6540
 *   pulseGenerator                            eden/Eden.cpp:3798-3826
 *   sineGenerator, rampGenerator (LEMS)       LEMS_CoreComponents.inc.xml:430-458, 489-521, eden/Eden.cpp:3107-3133
 *   voltageClamp, voltageClampTriple (LEMS)   LEMS_CoreComponents.inc.xml:555-620
 *   timedSynapticInput                        eden/Eden.cpp:3759-3790, 3859-3871
 *   point neurons (LEMS): izhikevich2007Cell, iafTauCell, iafTauRefCell,
 *   iafCell, iafRefCell, adExIaFCell          LEMS_CoreComponents.inc.xml:957-1240, eden/Eden.cpp:6821-6914
 *   threshold crossing + spike send           eden/Eden.cpp:6247-6252, 3946-3995
 *   spike-list / generator sources            eden/Eden.cpp:6738-6790 (their steps come with the model)
 *   trajectory / event loggers                eden/Eden.cpp:11555-11635
 *
 * Its parity with the reference itself is pinned by tests/test_oracle_vs_reference.py
 * against fixtures produced by the reference simulator built from its own sources.
 */
#include <math.h>
/* The arithmetic type: IEEE single precision, as the reference's generated
 * kernels compute; building with -DEDEN_PORT_DOUBLE gives the same loop in
 * double precision (eden_port_run then still takes and returns the float
 * model and records), the FP64 reference the single-precision results'
 * errors are stated against. */
#ifdef EDEN_PORT_DOUBLE
typedef double real;
#define R(x) x
#define EXP exp
#define LOG log
#define SIN sin
#define POW pow
#else
typedef float real;
#define R(x) x##f
#define EXP expf
#define LOG logf
#define SIN sinf
#define POW powf
#endif
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/eden_gpu.h"

/* The per-step functions also compile as CUDA device code: the GPU build
 * (oracle/gpu64/eden_port_gpu.cu, double precision) runs this same source,
 * one thread per cell, as the FP64 GPU oracle. */
#ifdef __CUDACC__
#define PORT_FN __host__ __device__
#else
#define PORT_FN
#endif

/* ---- RNG: Thomas Wang's 64-bit integer hash, as used by randof ---------- */
static PORT_FN uint64_t hash64shift(uint64_t key) {
    key = (~key) + (key << 21);
    key = key ^ (key >> 24);
    key = (key + (key << 3)) + (key << 8);
    key = key ^ (key >> 14);
    key = (key + (key << 2)) + (key << 4);
    key = key ^ (key >> 28);
    key = key + (key << 31);
    return key;
}

static PORT_FN real randof(real x, int64_t work_item, int64_t instance, int64_t step, int invocation_id) {
    uint64_t hi = ((uint64_t)work_item << 24) | ((uint64_t)instance & ((1ULL << 24) - 1));
    uint64_t lo = ((uint64_t)(int64_t)invocation_id << 40) | ((uint64_t)step & ((1ULL << 40) - 1));
    uint64_t sample = hash64shift(hash64shift(lo) ^ hi);
    const int scale = 1 << 23;
    real r = (real)(sample % (uint64_t)scale) / (real)scale;
    return x * r;
}

static PORT_FN real rate_value(int kind, real r, real mid, real s, real v) {
    switch (kind) {
        case EDEN_RATE_EXP: return r * EXP((v - mid) / s);
        case EDEN_RATE_EXPLINEAR:
            return r * ((v == mid) ? R(1.0) : (((v - mid) / s) / (R(1.0) - EXP(-(v - mid) / s))));
        case EDEN_RATE_FIXED: return r;
        default: return r / (R(1.0) + EXP((mid - v) / s));
    }
}

typedef struct {
    const EdenGpuModel *m;
    int64_t n_target;
    /* double-buffered state */
    real *v[2], *gate[2], *izh_u[2], *izh_s[2];
    real *syn_a[2], *syn_b[2], *syn_pend[2];
    real *syn_R[2], *syn_U[2];          /* blockingPlasticSynapse plasticity state */
    unsigned char *trig[2];
    real *pois_ts[2], *pois_isi[2], *pois_a[2], *pois_b[2];
    real *timed_a[2], *timed_b[2];      /* timedSynapticInput synapse states */
    int64_t *timed_cur;                 /* next listed step of each timed input */
    int64_t *timed_tgt_off;             /* [n_target + 1] timed inputs by target */
    int64_t *timed_order;               /* inputs in target order */
    int64_t *gap_off, *gap_order;       /* gap-junction ends by target, model order within one */
    int64_t *gr_off, *gr_order;         /* gradedSynapse ends likewise */
    real *gr_s[2];                      /* their state s */
    unsigned char *spiked[2];           /* event-logger slot per source */
    real *diag;
    int64_t *gate_off;                  /* [n_chan + 1] */
    int64_t *syn_off, *pois_off, *pulse_off, *wave_off, *clamp_off; /* [n_target + 1] */
    int64_t *fan_off, *fan_syn;         /* CSR source -> synapses */
    int32_t *order;                     /* per-cell DFS post-order, local ids */
    int32_t *src_of_target;             /* source id detecting at a target, or -1 */
    int64_t *syn_fire_count;
} Port;

static int64_t *csr_by_key(const int32_t *key, int64_t n, int64_t nkeys) {
    int64_t *off = (int64_t *)calloc((size_t)nkeys + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) off[key[i] + 1]++;
    for (int64_t k = 0; k < nkeys; k++) off[k + 1] += off[k];
    return off;
}

/* Depth-first post-order from the root, children in increasing index order
 * (BackwardEuler::GetOrderLists, eden/Eden.cpp:4411-4473). */
static void dfs_postorder(const int32_t *parent, int n, int32_t *order) {
    int *child_off = (int *)calloc((size_t)n + 1, sizeof(int));
    int *children = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 1; i < n; i++) child_off[parent[i] + 1]++;
    for (int i = 0; i < n; i++) child_off[i + 1] += child_off[i];
    int *fill = (int *)calloc((size_t)n + 1, sizeof(int));
    for (int i = 1; i < n; i++) children[child_off[parent[i]] + fill[parent[i]]++] = i;
    int *stack = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    int *next = (int *)calloc((size_t)n + 1, sizeof(int));
    int sp = 0, k = 0;
    if (n > 0) stack[sp++] = 0;
    while (sp > 0) {
        int u = stack[sp - 1];
        if (next[u] < child_off[u + 1] - child_off[u]) {
            stack[sp++] = children[child_off[u] + next[u]++];
        } else {
            order[k++] = u;
            sp--;
        }
    }
    free(child_off); free(children); free(fill); free(stack); free(next);
}

/* One step of a synapse's own state (a, b) with `fired` this step: the
 * exposure before the update -- conductance g and current i, or for the
 * current-based alphaCurrentSynapse its current with g = 0 -- and the next
 * state.  expOne as the reference's native code (eden/Eden.cpp:3424-3466);
 * the LEMS kinds by forward Euler of their TimeDerivatives, an OnEvent
 * assignment replacing the integrated value of the state it assigns
 * (LEMS_CoreComponents.inc.xml:85-180): expTwo (a = A, b = B), alpha
 * (a = A, b = g) and alphaCurrent (a = J, b = I). */
static inline PORT_FN void syn_dyn(const EdenGpuSynapseType *st, int init, int fired, real dt, real v, real a,
                                   real b, real *an, real *bn, real *g, real *i, real js) {
    const real e = (real)2.7182818284590451;
    switch (st->kind) {
    case EDEN_SYN_EXPONE:
        *g = a;
        *i = *g * (st->erev - v);
        *an = init ? a : (fired ? a + st->gbase : a - dt * (a / st->tau_decay));
        *bn = b;
        return;
    case EDEN_SYN_EXPONE_CURRENT:
        /* expCurrSynapse: I' = -I / tau_syn, I += weight on an event, the
         * current I (LEMS_CoreComponents.inc.xml:1858-1877) */
        *g = R(0.0);
        *i = a;
        *an = init ? a : (fired ? a + st->gbase : a + dt * (-a / st->tau_decay));
        *bn = b;
        return;
    case EDEN_SYN_ALPHA:
    case EDEN_SYN_ALPHA_CURRENT:
        if (st->kind == EDEN_SYN_ALPHA) {
            *g = b;
            *i = *g * (st->erev - v);
        } else {
            *g = R(0.0);
            *i = b;
        }
        if (init) {
            *an = R(0.0); *bn = R(0.0);
        } else {
            *an = fired ? a + st->gbase * st->weight_prop : a + dt * (-a / st->tau_decay);
            *bn = b + dt * ((e * a - b) / st->tau_decay);
        }
        return;
    default:
        /* expTwo; a blockingPlasticSynapse scales its conductance by the
         * voltage block 1 / (1 + ratio exp(-V / volt)) and each event's jump
         * by the plasticity factor js (LEMS_CoreComponents.inc.xml:231-352) */
        if (st->kind == EDEN_SYN_BLOCKING_PLASTIC && st->block_volt != 0.0f)
            *g = ((R(1.0) / (R(1.0) + (real)st->block_ratio * EXP(R(-1.0) * (v / (real)st->block_volt)))) * st->gbase) *
                 (b - a);
        else
            *g = st->gbase * (b - a);
        *i = *g * (st->erev - v);
        if (init) {
            *an = R(0.0); *bn = R(0.0);
        } else if (fired) {
            *an = a + st->weight_prop * js * st->waveform_factor;
            *bn = b + st->weight_prop * js * st->waveform_factor;
        } else {
            *an = a + dt * (-a / st->tau_rise);
            *bn = b + dt * (-b / st->tau_decay);
        }
        return;
    }
}

/* One synapse instance: trigger/pending logic, exposure, state update.
 * Returns the weighted current and conductance through *iw, *gw. */
static inline PORT_FN void synapse_step(const EdenGpuSynapseType *st, int init, real t, real dt,
                                int spike_in_raw, real delay, real pend, real *pend_next,
                                real a, real b, real *a_next, real *b_next, real v, real w,
                                real *iw, real *gw, int *fired, real pr, real pu, real *pr_next, real *pu_next) {
    int spike_now = 0;
    real next_next = pend;
    if (!init) {
        if (t <= pend && pend < t + dt) spike_now = 1;
        if (spike_in_raw) {
            real fresh = t + delay;
            if (t <= fresh && fresh < t + dt) spike_now = 1;
            if (next_next < t + dt && next_next < fresh) next_next = fresh;
        }
    }
    *pend_next = next_next;
    *fired = spike_now;
    /* a blockingPlasticSynapse's Tsodyks-Markram state, forward Euler, the
     * event assignments from the step's values overriding
     * (LEMS_CoreComponents.inc.xml:263-312) */
    real js = R(1.0);
    if (st->kind == EDEN_SYN_BLOCKING_PLASTIC && st->tau_rec > 0.0f) {
        const real p = st->release_prob;
        if (init) {
            *pr_next = R(1.0); *pu_next = p;
        } else if (spike_now) {
            js = pr * pu;
            *pr_next = pr * (R(1.0) - pu);
            *pu_next = st->tau_fac > 0.0f ? pu + p * (R(1.0) - pu) : p;
        } else {
            *pr_next = pr + dt * ((R(1.0) - pr) / (real)st->tau_rec);
            *pu_next = st->tau_fac > 0.0f ? pu + dt * ((p - pu) / (real)st->tau_fac) : p;
        }
    }
    real g, i;
    syn_dyn(st, init, spike_now, dt, v, a, b, a_next, b_next, &g, &i, js);
    *iw = i * w;
    *gw = g * w;
}

/* Poisson-driven synapse: the spiker fires its own synapse in the same step. */
static inline PORT_FN void poisson_step(const Port *P, int cur, int64_t k, int init, real dt, int64_t step,
                                real v, real *iw, real *gw) {
    const EdenGpuModel *m = P->m;
    int nxt = cur ^ 1;
    real rate = m->pois_rate[k];
    real avg_isi = R(1.0) / rate;
    int64_t work_item = (int64_t)m->src_cell_seed[m->pois_src[k]];
    int64_t inst = m->pois_instance[k];
    const int base = m->pois_rng_base ? m->pois_rng_base[k] : 0;
    real ts = P->pois_ts[cur][k], isi = P->pois_isi[cur][k];
    int fired = 0;
    if (init) {
        P->pois_ts[nxt][k] = R(0.0);
        P->pois_isi[nxt][k] = (-avg_isi) * LOG(R(1.0) - randof(R(1.0), work_item, inst, step, base));
    } else {
        P->pois_ts[nxt][k] = ts + dt * R(1.0);
        P->pois_isi[nxt][k] = isi;
        if (ts > isi) {
            P->pois_ts[nxt][k] = R(0.0);
            P->pois_isi[nxt][k] = (-avg_isi) * LOG(R(1.0) - randof(R(1.0), work_item, inst, step, base + 1));
            fired = 1;
        }
    }
    const EdenGpuSynapseType *st = &m->syn_types[m->pois_type[k]];
    real g, i, an, bn;
    syn_dyn(st, init, fired, dt, v, P->pois_a[cur][k], P->pois_b[cur][k], &an, &bn, &g, &i, R(1.0));
    P->pois_a[nxt][k] = an;
    P->pois_b[nxt][k] = bn;
    *iw = i * m->pois_weight[k];
    *gw = g * m->pois_weight[k];
}

/* timedSynapticInput: its synapse fires in the listed steps (the first step
 * whose t + dt exceeds a spike time, eden/Eden.cpp:3759-3790, 3859-3871;
 * computed at lowering), with the synapse's own dynamics as in poisson_step. */
static inline PORT_FN void timed_input_step(const Port *P, int cur, int64_t k, int init, real dt, int64_t step,
                                            real v, real *iw, real *gw) {
    const EdenGpuModel *m = P->m;
    int nxt = cur ^ 1;
    int fired = 0;
    if (!init) {
        int64_t c = P->timed_cur[k];
        if (c < m->timed_off[k + 1] && m->timed_step[c] == step) {
            fired = 1;
            P->timed_cur[k] = c + 1;
        }
    }
    const EdenGpuSynapseType *st = &m->syn_types[m->timed_type[k]];
    real g, i, an, bn;
    syn_dyn(st, init, fired, dt, v, P->timed_a[cur][k], P->timed_b[cur][k], &an, &bn, &g, &i, R(1.0));
    P->timed_a[nxt][k] = an;
    P->timed_b[nxt][k] = bn;
    *iw = i * m->timed_weight[k];
    *gw = g * m->timed_weight[k];
}

/* Synapse + input currents into one target (in the reference's order:
 * inputs then synapses are separate totals, each synapse type a block). */
static PORT_FN void target_currents(Port *P, int cur, int64_t tgt, int init, real t, real dt, int64_t step,
                            real v, real *I_in, real *G_in, real *I_syn, real *G_syn) {
    const EdenGpuModel *m = P->m;
    int nxt = cur ^ 1;
    real Iin = R(0.0), Gin = R(0.0), Isyn = R(0.0), Gsyn = R(0.0);
    /* pulses */
    if (P->pulse_off[tgt + 1] > P->pulse_off[tgt]) {
        real Ip = R(0.0);
        for (int64_t k = P->pulse_off[tgt]; k < P->pulse_off[tgt + 1]; k++) {
            real s = m->pulse_start[k];
            if (s <= t && t <= s + m->pulse_duration[k]) Ip += m->pulse_amplitude[k] * m->pulse_weight[k];
        }
        Iin += Ip;
    }
    /* sine and ramp generators: each adds its weighted current at once, the
     * value its OnConditions assign at this step's time (OnStart's in the
     * initialisation passes) */
    for (int64_t k = P->wave_off[tgt]; k < P->wave_off[tgt + 1]; k++) {
        const float *p = m->wave_params + (int64_t)EDEN_WAVE_PARAMS * k;
        const real del = p[0], dur = p[1];
        real i;
        if (m->wave_shape[k] == EDEN_WAVE_SINE) {
            const real amp = p[2], period = p[3], phase = p[4];
            if (init || t < del) i = R(0.0);
            else if (t < dur + del) i = (R(1.0) * amp) * SIN(phase + ((R(2.0) * R(3.14159265)) * (t - del)) / period);
            else i = R(0.0);
        } else {
            const real start = p[2], finish = p[3], base = p[4];
            if (init) i = base;
            else if (t < del) i = R(1.0) * base;
            else if (t < dur + del) i = R(1.0) * (start + ((finish - start) * (t - del)) / dur);
            else i = R(1.0) * base;
        }
        Iin += i * (real)m->wave_weight[k];
    }
    /* voltage clamps: the target of the phase the step's time is in (the
     * OnConditions in order, the last that holds assigns), against the
     * potential at the start of the step; none in the initialisation passes */
    for (int64_t k = P->clamp_off[tgt]; k < P->clamp_off[tgt + 1]; k++) {
        const float *p = m->clamp_params + (int64_t)EDEN_CLAMP_PARAMS * k;
        const real del = p[0], dur = p[1];
        const real tv = (t > dur + del) ? (real)p[4] : (t < del) ? (real)p[2] : (real)p[3];
        if (!init && tv == tv) Iin += ((R(1.0) * (tv - v)) / (real)p[5]) * (real)m->clamp_weight[k];
    }
    /* Poisson inputs, one block per synapse type run */
    int64_t k = P->pois_off[tgt];
    while (k < P->pois_off[tgt + 1]) {
        int type = m->pois_type[k];
        real Ia = R(0.0), Ga = R(0.0);
        for (; k < P->pois_off[tgt + 1] && m->pois_type[k] == type; k++) {
            real iw, gw;
            poisson_step(P, cur, k, init, dt, step, v, &iw, &gw);
            Ia += iw; Ga += gw;
        }
        Iin += Ia; Gin += Ga;
    }
    /* timed inputs, one block per synapse type run */
    int64_t q = P->timed_tgt_off[tgt];
    while (q < P->timed_tgt_off[tgt + 1]) {
        int type = m->timed_type[P->timed_order[q]];
        real Ia = R(0.0), Ga = R(0.0);
        for (; q < P->timed_tgt_off[tgt + 1] && m->timed_type[P->timed_order[q]] == type; q++) {
            real iw, gw;
            timed_input_step(P, cur, P->timed_order[q], init, dt, step, v, &iw, &gw);
            Ia += iw; Ga += gw;
        }
        Iin += Ia; Gin += Ga;
    }
    /* connection synapses, one block per synapse type */
    int64_t s = P->syn_off[tgt];
    while (s < P->syn_off[tgt + 1]) {
        int type = m->syn_type[s];
        const EdenGpuSynapseType *st = &m->syn_types[type];
        real Ia = R(0.0), Ga = R(0.0);
        for (; s < P->syn_off[tgt + 1] && m->syn_type[s] == type; s++) {
            int in = 0;
            if (!init) {
                in = P->trig[cur][s] != 0;
                P->trig[cur][s] = 0;
            }
            real iw, gw;
            int fired;
            synapse_step(st, init, t, dt, in, m->syn_delay[s], P->syn_pend[cur][s], &P->syn_pend[nxt][s],
                         P->syn_a[cur][s], P->syn_b[cur][s], &P->syn_a[nxt][s], &P->syn_b[nxt][s],
                         v, m->syn_weight[s], &iw, &gw, &fired, P->syn_R[cur][s], P->syn_U[cur][s],
                         &P->syn_R[nxt][s], &P->syn_U[nxt][s]);
            if (fired) P->syn_fire_count[s]++;
            Ia += iw; Ga += gw;
        }
        Isyn += Ia; Gsyn += Ga;
    }
    /* gap junctions: each end adds (g (V_peer - V)) w with the peer's
     * potential at the step's start, and no conductance term
     * (eden/Eden.cpp:3407-3422 exposure, 3689-3704 Vpeer, 3708-3710 sum) */
    if (P->gap_off[tgt] < P->gap_off[tgt + 1] || P->gr_off[tgt] < P->gr_off[tgt + 1]) {
        real Ia = R(0.0);
        for (int64_t q = P->gap_off[tgt]; q < P->gap_off[tgt + 1]; q++) {
            const int64_t k = P->gap_order[q];
            Ia += ((real)m->gap_conductance[k] * (P->v[cur][m->gap_peer[k]] - v)) * (real)m->gap_weight[k];
        }
        /* gradedSynapse ends (LEMS_CoreComponents.inc.xml:38-80): inf and tau
         * from the peer's potential, i = conductance s (erev - V) from the
         * step's s, s' = (inf - s) / tau by forward Euler while 1 - inf >
         * 1e-4, else s = inf; s = 0 at the initialisation steps */
        for (int64_t q = P->gr_off[tgt]; q < P->gr_off[tgt + 1]; q++) {
            const int64_t k = P->gr_order[q];
            const float *p = m->graded_params + (int64_t)EDEN_GRADED_PARAMS * k;
            const real s = P->gr_s[cur][k];
            const real inf = R(1.0) / (R(1.0) + EXP(((real)p[3] - P->v[cur][m->graded_peer[k]]) / (real)p[1]));
            const real tau = (R(1.0) - inf) / (real)p[2];
            Ia += (((real)p[0] * s) * ((real)p[4] - v)) * (real)m->graded_weight[k];
            real sn = R(0.0);
            if (!init) {
                sn = s + dt * ((R(1.0) - inf) > (real)1e-4 ? (inf - s) / tau : R(0.0));
                if ((R(1.0) - inf) < (real)1e-4) sn = inf;
            }
            P->gr_s[cur ^ 1][k] = sn;
        }
        Isyn += Ia;
    }
    *I_in = Iin; *G_in = Gin; *I_syn = Isyn; *G_syn = Gsyn;
}

static PORT_FN void send_spike(Port *P, int nxt, int32_t src) {
    for (int64_t e = P->fan_off[src]; e < P->fan_off[src + 1]; e++) {
#ifdef __CUDA_ARCH__
        ((volatile unsigned char *)P->trig[nxt])[P->fan_syn[e]] = 1;  /* every writer stores 1 */
#else
        __atomic_store_n(&P->trig[nxt][P->fan_syn[e]], (unsigned char)1, __ATOMIC_RELAXED);
#endif
    }
    P->spiked[nxt][src] = 1;
}

static PORT_FN void phys_cell_step(Port *P, int cur, int32_t cell, int init, real t, real dt, int64_t step) {
    const EdenGpuModel *m = P->m;
    int nxt = cur ^ 1;
    int32_t c0 = m->phys_comp_off[cell], c1 = m->phys_comp_off[cell + 1];
    const real *V = P->v[cur];
    real *Vn = P->v[nxt];
    const int fwd = m->cable_solver == EDEN_CABLE_FWD_EULER;
    if (fwd && !init) {
        /* forward Euler: each compartment's axial current (V_adj - V) / R
         * summed over its neighbours in ascending order -- the parent, then
         * the children (eden/Eden.cpp:4969-4990, R_Axial of the higher index
         * of the pair) -- into diag.  Visiting the compartments in ascending
         * order adds, for each one, its parent's term at its own visit and
         * its children's at theirs, later and in ascending order. */
        for (int32_t c = c0; c < c1; c++) P->diag[c] = R(0.0);
        for (int32_t c = c0 + 1; c < c1; c++) {
            int32_t j = c0 + m->comp_parent[c];
            real Rr = m->comp_r_axial[c > j ? c : j];
            P->diag[c] += (V[j] - V[c]) / Rr;
            P->diag[j] += (V[c] - V[j]) / Rr;
        }
    }
    for (int32_t c = c0; c < c1; c++) {
        real A = m->comp_area[c], Vc = V[c];
        real Ich = R(0.0), Gch = R(0.0);
        for (int32_t ch = m->comp_chan_off[c]; ch < m->comp_chan_off[c + 1]; ch++) {
            const EdenGpuChannelType *ct = &m->chan_types[m->chan_type[ch]];
            real fopen = R(1.0);
            int64_t go = P->gate_off[ch];
            for (int g = 0; g < ct->n_gates; g++) {
                real q = P->gate[cur][go + g];
                /* tau and inf from the rates unless the gate kind has its
                 * own timeCourse / steadyState (eden/Eden.cpp:5290-5375) */
                const int gk = ct->gate_kind[g];
                if (gk == EDEN_GATE_INSTANTANEOUS) {
                    /* no state: the steady state at this step's V (eden/Eden.cpp:5268-5282) */
                    const real x = rate_value(ct->inf_kind[g], ct->inf_rate[g], ct->inf_mid[g], ct->inf_scale[g], Vc);
                    P->gate[nxt][go + g] = x;
                    for (int r = 0; r < ct->gate_instances[g]; r++) fopen = fopen * x;
                    continue;
                }
                real alpha = R(0.0), beta = R(0.0);
                if (gk != EDEN_GATE_TAUINF) {
                    alpha = rate_value(ct->fwd_kind[g], ct->fwd_rate[g], ct->fwd_mid[g], ct->fwd_scale[g], Vc);
                    beta = rate_value(ct->rev_kind[g], ct->rev_rate[g], ct->rev_mid[g], ct->rev_scale[g], Vc);
                }
                real tau, inf;
                if (gk == EDEN_GATE_TAUINF || gk == EDEN_GATE_RATESTAU || gk == EDEN_GATE_RATESTAUINF)
                    tau = rate_value(ct->tau_kind[g], ct->tau_rate[g], ct->tau_mid[g], ct->tau_scale[g], Vc);
                else
                    tau = R(1.0) / (alpha + beta);
                if (gk == EDEN_GATE_TAUINF || gk == EDEN_GATE_RATESINF || gk == EDEN_GATE_RATESTAUINF)
                    inf = rate_value(ct->inf_kind[g], ct->inf_rate[g], ct->inf_mid[g], ct->inf_scale[g], Vc);
                else
                    inf = alpha / (alpha + beta);
                real qn;
                if (init) {
                    qn = inf;
                } else {
                    real tau_factor = (dt * ct->q10[g]) / tau;
                    real blend = EXP(-tau_factor);
                    qn = blend * q + (R(1.0) - blend) * inf;
                    if (!(qn > R(1e-6))) qn = R(1e-6);
                    if (!(qn < (real)(1 - 1e-6))) qn = (real)(1 - 1e-6);
                }
                P->gate[nxt][go + g] = qn;
                for (int r = 0; r < ct->gate_instances[g]; r++) fopen = fopen * q;
            }
            real Gscaled = m->chan_gbase[ch] * fopen;
            real iD = Gscaled * (m->chan_erev[ch] - Vc) * R(1e-5);
            real gD = Gscaled * R(1e-5);
            Ich += iD * A;
            Gch += gD * A;
        }
        real Iin, Gin, Isyn, Gsyn;
        target_currents(P, cur, c, init, t, dt, step, Vc, &Iin, &Gin, &Isyn, &Gsyn);
        real I = Ich + Iin + Isyn;
        real G = Gch + Gin + Gsyn;
        if (fwd) {
            /* V_next = V + dt (I + I_axial) / C (eden/Eden.cpp:6092-6094) */
            Vn[c] = init ? Vc : Vc + (dt * (I + P->diag[c])) / m->comp_c[c];
            continue;
        }
        P->diag[c] = R(1.0) * (G / m->comp_c[c]) + m->comp_inv_rc[c];
        Vn[c] = init ? Vc : Vc + (dt * (I + (Vc * G))) / m->comp_c[c];
    }
    if (!init && !fwd) {
        int32_t n = c1 - c0;
        const int32_t *ord = P->order + c0;
        const int32_t *par = m->comp_parent + c0;
        const float *R = m->comp_r_axial + c0, *C = m->comp_c + c0;
        real *D = P->diag + c0, *X = Vn + c0;
        for (int32_t k = 0; k < n; k++) D[k] = R(1.0) + D[k] * dt;
        for (int32_t k = 0; k < n - 1; k++) {
            int32_t i = ord[k], j = par[i];
            int32_t idx = i > j ? i : j;
            real Rr = R[idx];
            real Ui = -dt / (Rr * C[i]);
            real Uj = -dt / (Rr * C[j]);
            real ratio = Uj / D[i];
            D[j] -= ratio * Ui;
            X[j] -= ratio * X[i];
        }
        int32_t r = ord[n - 1];
        X[r] = X[r] / D[r];
        for (int32_t k = n - 2; k >= 0; k--) {
            int32_t i = ord[k], j = par[i];
            int32_t idx = i > j ? i : j;
            real Rr = R[idx];
            real Ui = -dt / (Rr * C[i]);
            X[i] = (X[i] - Ui * X[j]) / D[i];
        }
    }
    for (int32_t c = c0; c < c1; c++) {
        int32_t src = P->src_of_target[c];
        if (src < 0) continue;
        real thr = m->src_threshold[src];
        if (V[c] < thr && thr < Vn[c]) send_spike(P, nxt, src);
    }
}

/* A point neuron for one step (LEMS_CoreComponents.inc.xml: izhikevich2007Cell
 * 1140-1187, iafTauCell 957-983, iafTauRefCell 985-1021, iafCell 1023-1056,
 * iafRefCell 1058-1095, adExIaFCell 1189-1240, izhikevichCell), with the semantics of the
 * reference's LEMS code (eden/Eden.cpp:2832-2994): forward Euler from the now
 * state, OnCondition assignments (from now values) overriding, OnStart in the
 * initialisation passes.  State u is izhikevich u / adEx w, s the last spike
 * time. */
static PORT_FN void izh_step(Port *P, int cur, int32_t k, int init, real t, real dt, int64_t step) {
    const EdenGpuModel *m = P->m;
    int nxt = cur ^ 1;
    int64_t tgt = (int64_t)m->n_comp + k;
    const float *p = m->izh_params + EDEN_POINT_PARAMS * (int64_t)k;
    int kind = m->izh_kind ? m->izh_kind[k] : EDEN_POINT_IZH2007;
    real v = P->v[cur][tgt], u = P->izh_u[cur][k], s = P->izh_s[cur][k];
    real Iin, Gin, Isyn, Gsyn;
    target_currents(P, cur, tgt, init, t, dt, step, v, &Iin, &Gin, &Isyn, &Gsyn);
    real iext = Isyn + Iin;
    real vn = v, un = u, sn = s;
    int spike = 0;
    if (kind == EDEN_POINT_IZH2007) {
        real C = p[0], v0 = p[1], kk = p[2], vr = p[3], vt = p[4], vpeak = p[5];
        real a = p[6], b = p[7], c = p[8], d = p[9];
        real iMemb = ((kk * (v - vr)) * R(1e-3)) * (v - vt) + iext - u;
        if (init) {
            vn = v0;
            un = R(0.0);
        } else {
            real dv = iMemb / C;
            vn = v + dt * dv;
            real du = (a * ((b * (v - vr)) - u)) * R(1e-3);
            un = u + dt * du * R(1e3);
            if (v > vpeak) {
                vn = c;
                un = u + d;
                spike = 1;
            }
        }
    } else if (kind == EDEN_POINT_IAF_TAU || kind == EDEN_POINT_IAF_TAU_REF) {
        /* no synaptic current: v' = (leakReversal - v) / tau */
        int ref = kind == EDEN_POINT_IAF_TAU_REF;
        real EL = p[0], tau = p[1], thresh = p[2], reset = p[3], refract = ref ? p[4] : R(0.0);
        if (init) {
            vn = EL;
            if (ref) sn = t - refract;
        } else {
            int active = !ref || t > s + refract;
            real rate = active ? (EL - v) / tau : R(0.0);
            vn = v + dt * rate;
            if (v > thresh && active) {
                if (ref) sn = t;
                vn = reset;
                spike = 1;
            }
        }
    } else if (kind == EDEN_POINT_IAF || kind == EDEN_POINT_IAF_REF) {
        int ref = kind == EDEN_POINT_IAF_REF;
        real C = p[0], gL = p[1], EL = p[2], thresh = p[3], reset = p[4], refract = ref ? p[5] : R(0.0);
        if (init) {
            vn = EL;
            if (ref) sn = t - refract;
        } else {
            real iMemb = gL * (EL - v) + iext;
            int active = !ref || t > s + refract;
            real rate = active ? iMemb / C : R(0.0);
            vn = v + dt * rate;
            if (v > thresh && active) {
                if (ref) sn = t;
                vn = reset;
                spike = 1;
            }
        }
    } else if (kind == EDEN_POINT_FN) {
        /* fitzHughNagumoCell: forward Euler with SEC = 1e6 us; V and W keep
         * their initial values through the initialisation passes */
        const real SEC = R(1.0e6);
        if (!init) {
            vn = v + dt * ((((v - POW(v, R(3.0)) / R(3.0)) - u) + (real)p[0]) / SEC);
            un = u + dt * ((R(0.08) * ((v + R(0.7)) - R(0.8) * u)) / SEC);
        }
    } else if (kind == EDEN_POINT_IZH_DL) {
        /* izhikevichCell: forward Euler with MSEC = 1000 us, MVOLT = 1 mV */
        real v0 = p[0], thresh = p[1], a = p[2], b = p[3], c = p[4], d = p[5];
        const real MV = R(1.0), MS = R(1000.0);
        if (init) {
            vn = v0;
            un = (v0 * b) / MV;
        } else {
            real dv = ((R(0.04) * ((v * v) / MV) + R(5.0) * v) + ((R(140.0) - u) + iext) * MV) / MS;
            real du = (a * ((b * v) / MV - u)) / MS;
            vn = v + dt * dv;
            un = u + dt * du;
            if (v > thresh) {
                vn = c * MV;
                un = u + d;
                spike = 1;
            }
        }
    } else { /* EDEN_POINT_ADEX */
        real C = p[0], gL = p[1], EL = p[2], VT = p[3], thresh = p[4], reset = p[5];
        real delT = p[6], tauw = p[7], refract = p[8], a = p[9], b = p[10];
        if (init) {
            vn = EL;
            un = R(0.0);
            sn = t - refract;
        } else {
            real iMemb = (R(-1.0) * gL) * (v - EL) + (gL * delT) * EXP((v - VT) / delT) - u + iext;
            int active = t > s + refract;
            real rate = active ? iMemb / C : R(0.0);
            vn = v + dt * rate;
            un = u + dt * ((a * (v - EL) - u) / tauw);
            if (v > thresh && active) {
                sn = t;
                vn = reset;
                un = u + b;
                spike = 1;
            }
        }
    }
    P->v[nxt][tgt] = vn;
    P->izh_u[nxt][k] = un;
    P->izh_s[nxt][k] = sn;
    int32_t src = P->src_of_target[tgt];
    if (spike && src >= 0) send_spike(P, nxt, src);
}

/*
 * Run the model for `n_steps` non-initialisation steps (after the 4
 * initialisation passes), recording V of `trace_target` (or, for an entry
 * -2 - g, the state of gate g in channel-instance order) at every step's
 * output phase into trace[step][col] and every logged spike as
 * (source, logging step).  Returns 0 or a negative code.
 */
/* Host set-up of the loop's state (initial values, CSR tables, Hines
 * orders); also used by the GPU build, which mirrors it to the device. */
static void port_setup(Port *PP, const EdenGpuModel *m) {
    Port P;
    memset(&P, 0, sizeof(P));
    P.m = m;
    int64_t nt = (int64_t)m->n_comp + m->n_izh;
    P.n_target = nt;
    int64_t n_chan = m->comp_chan_off[m->n_comp];
    P.gate_off = (int64_t *)calloc((size_t)n_chan + 1, sizeof(int64_t));
    for (int64_t ch = 0; ch < n_chan; ch++)
        P.gate_off[ch + 1] = P.gate_off[ch] + m->chan_types[m->chan_type[ch]].n_gates;
    int64_t n_gate = P.gate_off[n_chan];
    int64_t ns = m->n_syn, np = m->n_pois;
    for (int b = 0; b < 2; b++) {
        P.v[b] = (real *)calloc((size_t)nt + 1, sizeof(real));
        P.gate[b] = (real *)calloc((size_t)n_gate + 1, sizeof(real));
        P.izh_u[b] = (real *)calloc((size_t)m->n_izh + 1, sizeof(real));
        P.izh_s[b] = (real *)calloc((size_t)m->n_izh + 1, sizeof(real));
        P.syn_a[b] = (real *)calloc((size_t)ns + 1, sizeof(real));
        P.syn_b[b] = (real *)calloc((size_t)ns + 1, sizeof(real));
        P.syn_pend[b] = (real *)calloc((size_t)ns + 1, sizeof(real));
        P.syn_R[b] = (real *)calloc((size_t)ns + 1, sizeof(real));
        P.syn_U[b] = (real *)calloc((size_t)ns + 1, sizeof(real));
        for (int64_t q = 0; q < ns; q++) {
            P.syn_R[b][q] = R(1.0);
            P.syn_U[b][q] = m->syn_types[m->syn_type[q]].release_prob;
        }
        P.trig[b] = (unsigned char *)calloc((size_t)ns + 1, 1);
        P.pois_ts[b] = (real *)calloc((size_t)np + 1, sizeof(real));
        P.pois_isi[b] = (real *)calloc((size_t)np + 1, sizeof(real));
        P.pois_a[b] = (real *)calloc((size_t)np + 1, sizeof(real));
        P.pois_b[b] = (real *)calloc((size_t)np + 1, sizeof(real));
        P.spiked[b] = (unsigned char *)calloc((size_t)m->n_src + 1, 1);
    }
    for (int b = 0; b < 2; b++) {
        P.timed_a[b] = (real *)calloc((size_t)m->n_timed + 1, sizeof(real));
        P.timed_b[b] = (real *)calloc((size_t)m->n_timed + 1, sizeof(real));
    }
    P.timed_cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m->n_timed + 1));
    for (int64_t k = 0; k < m->n_timed; k++) P.timed_cur[k] = m->timed_off[k];
    P.timed_tgt_off = csr_by_key(m->timed_target, m->n_timed, nt);
    P.timed_order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m->n_timed + 1));
    {
        /* stable by target, then type (input order within a type) */
        int64_t *fill = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
        for (int pass = 0; pass < 1; pass++) {
            for (int64_t k = 0; k < m->n_timed; k++) {
                int32_t t = m->timed_target[k];
                P.timed_order[P.timed_tgt_off[t] + fill[t]++] = k;
            }
        }
        free(fill);
        for (int64_t t = 0; t < nt; t++) {  /* insertion sort by type inside each target */
            for (int64_t i = P.timed_tgt_off[t] + 1; i < P.timed_tgt_off[t + 1]; i++) {
                int64_t x = P.timed_order[i], j = i - 1;
                while (j >= P.timed_tgt_off[t] && m->timed_type[P.timed_order[j]] > m->timed_type[x]) {
                    P.timed_order[j + 1] = P.timed_order[j];
                    j--;
                }
                P.timed_order[j + 1] = x;
            }
        }
    }
    P.diag = (real *)calloc((size_t)m->n_comp + 1, sizeof(real));
    P.syn_fire_count = (int64_t *)calloc((size_t)ns + 1, sizeof(int64_t));
    /* initial state: V0, izhikevich v0, pending spikes at -inf (eden/Eden.cpp:9081-9094) */
    for (int b = 0; b < 2; b++) {
        for (int32_t c = 0; c < m->n_comp; c++) P.v[b][c] = m->comp_v0[c];
        for (int32_t k = 0; k < m->n_izh; k++) {
            /* the value OnStart gives V */
            int kind = m->izh_kind ? m->izh_kind[k] : EDEN_POINT_IZH2007;
            int f = (kind == EDEN_POINT_IZH2007 || kind == EDEN_POINT_FN) ? 1
                    : (kind == EDEN_POINT_IAF_TAU || kind == EDEN_POINT_IAF_TAU_REF || kind == EDEN_POINT_IZH_DL) ? 0 : 2;
            P.v[b][m->n_comp + k] = m->izh_params[EDEN_POINT_PARAMS * (int64_t)k + f];
        }
        for (int64_t s = 0; s < ns; s++) P.syn_pend[b][s] = -INFINITY;
    }
    P.syn_off = csr_by_key(m->syn_target, ns, nt);
    P.pois_off = csr_by_key(m->pois_target, np, nt);
    P.pulse_off = csr_by_key(m->pulse_target, m->n_pulse, nt);
    P.wave_off = csr_by_key(m->wave_target, m->n_wave, nt);
    P.clamp_off = csr_by_key(m->clamp_target, m->n_clamp, nt);
    P.fan_off = csr_by_key(m->syn_src, ns, m->n_src);
    P.gr_off = csr_by_key(m->graded_target, m->n_graded, nt);
    P.gr_order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m->n_graded + 1));
    {
        int64_t *fill = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
        for (int64_t k = 0; k < m->n_graded; k++) {
            int32_t t = m->graded_target[k];
            P.gr_order[P.gr_off[t] + fill[t]++] = k;
        }
        free(fill);
    }
    for (int b = 0; b < 2; b++) P.gr_s[b] = (real *)calloc((size_t)m->n_graded + 1, sizeof(real));
    P.gap_off = csr_by_key(m->gap_target, m->n_gap, nt);
    P.gap_order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m->n_gap + 1));
    {
        int64_t *fill = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
        for (int64_t k = 0; k < m->n_gap; k++) {
            int32_t t = m->gap_target[k];
            P.gap_order[P.gap_off[t] + fill[t]++] = k;
        }
        free(fill);
    }
    P.fan_syn = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ns + 1));
    {
        int64_t *fill = (int64_t *)calloc((size_t)m->n_src + 1, sizeof(int64_t));
        for (int64_t s = 0; s < ns; s++) {  /* connection order = synapse order */
            int32_t src = m->syn_src[s];
            P.fan_syn[P.fan_off[src] + fill[src]++] = s;
        }
        free(fill);
    }
    P.order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m->n_comp + 1));
    for (int32_t cell = 0; cell < m->n_phys; cell++) {
        int32_t c0 = m->phys_comp_off[cell], c1 = m->phys_comp_off[cell + 1];
        dfs_postorder(m->comp_parent + c0, c1 - c0, P.order + c0);
    }
    P.src_of_target = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nt + 1));
    for (int64_t t = 0; t < nt; t++) P.src_of_target[t] = -1;
    for (int32_t s = 0; s < m->n_src; s++)
        if (m->src_target[s] >= 0) P.src_of_target[m->src_target[s]] = s;  /* -1: a spike list or generator */
    *PP = P;
}

static void port_free(Port *P) {
    for (int b = 0; b < 2; b++) {
        free(P->v[b]); free(P->gate[b]); free(P->izh_u[b]); free(P->izh_s[b]); free(P->syn_a[b]); free(P->syn_b[b]);
        free(P->syn_pend[b]); free(P->syn_R[b]); free(P->syn_U[b]); free(P->trig[b]); free(P->pois_ts[b]); free(P->pois_isi[b]);
        free(P->pois_a[b]); free(P->pois_b[b]); free(P->spiked[b]); free(P->timed_a[b]); free(P->timed_b[b]);
    }
    free(P->diag); free(P->syn_fire_count); free(P->gate_off); free(P->syn_off); free(P->pois_off);
    free(P->pulse_off); free(P->wave_off); free(P->clamp_off); free(P->fan_off); free(P->fan_syn); free(P->order); free(P->src_of_target);
    free(P->timed_cur); free(P->timed_tgt_off); free(P->timed_order); free(P->gap_off); free(P->gap_order);
    free(P->gr_off); free(P->gr_order); free(P->gr_s[0]); free(P->gr_s[1]);
}

/* Wall-clock marks for timing a stretch of a run (the CPU timings beside
 * the GPU's): the time at the start of step eden_port_mark_step (before its
 * output phase) and at the end of the run, in seconds of one clock. */
int64_t eden_port_mark_step = INT64_MAX;
double eden_port_mark_s = 0.0, eden_port_end_s = 0.0;

static double wall_s(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

int eden_port_run(const EdenGpuModel *m, int64_t n_steps, int32_t n_trace, const int32_t *trace_target,
                  float *trace, int64_t spike_cap, int32_t *spike_src, int64_t *spike_step,
                  int64_t *n_spikes, int64_t *syn_fire_count, float *syn_final_pending, int32_t n_threads) {
    if (!m || m->abi_version != EDEN_GPU_ABI_VERSION) return EDEN_GPU_E_INVALID;
    Port P;
    port_setup(&P, m);
    const int64_t ns = m->n_syn;

#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    int cur = 0;
    double time = 0.0;
    const real dt = m->dt;
    int64_t nsp = 0;
    int rc = 0;
    int64_t last_step = n_steps;  /* steps 1..n_steps are the non-init ones */
    int64_t ext = 0;              /* next spike-source event */
    for (int64_t step = -3; step <= last_step; step++) {
        int init = step <= 0;
        if (step == eden_port_mark_step) eden_port_mark_s = wall_s();
        if (!init) {
            /* output phase: trajectory columns, then event slots read & clear */
            for (int32_t j = 0; j < n_trace; j++)  /* V of a target, or (-2 - g) gate g's state */
                trace[(step - 1) * n_trace + j] =
                    trace_target[j] >= 0 ? P.v[cur][trace_target[j]] : P.gate[cur][-2 - (int64_t)trace_target[j]];
            for (int32_t s = 0; s < m->n_src; s++) {
                if (P.spiked[cur][s]) {
                    if (nsp < spike_cap) {
                        spike_src[nsp] = s;
                        spike_step[nsp] = step;
                    } else {
                        rc = EDEN_GPU_E_RANGE;
                    }
                    nsp++;
                }
                P.spiked[cur][s] = 0;
            }
        }
        real t = (real)time;
        int32_t n_items = m->n_phys + m->n_izh;
#pragma omp parallel for schedule(static)
        for (int32_t item = 0; item < n_items; item++) {
            if (item < m->n_phys)
                phys_cell_step(&P, cur, item, init, t, dt, step);
            else
                izh_step(&P, cur, item - m->n_phys, init, t, dt, step);
        }
        /* sources with no target (spike lists, generators): the spikes this
         * step emits, logged at the next step like a cell's */
        while (ext < m->n_ext && m->ext_step[ext] <= step + 1) {
            if (m->ext_step[ext] == step + 1) send_spike(&P, cur ^ 1, m->ext_src[ext]);
            ext++;
        }
        if (!init) time += dt;
        cur ^= 1;
    }
    eden_port_end_s = wall_s();
    *n_spikes = nsp;
    if (syn_fire_count) memcpy(syn_fire_count, P.syn_fire_count, sizeof(int64_t) * (size_t)ns);
    if (syn_final_pending)
        for (int64_t s = 0; s < ns; s++) syn_final_pending[s] = (float)P.syn_pend[cur][s];
    port_free(&P);
    return rc;
}
