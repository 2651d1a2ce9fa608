/*
 * eden_gpu.h — C ABI of libeden_gpu.so, the GB300 (sm_103a) implementation of
 * EDEN's per-timestep simulation loop.
 *
 * The reference runs its step loop in eden/Eden.cpp:11488-11938: each step an
 * OpenMP loop calls one generated `doit()` per cell through the
 * `IterationCallback` C ABI (eden/Eden.cpp:64-76, called at 11856-11865), then
 * swaps the now/next state buffers (11935-11937).  This library replaces that
 * loop.  The host lowers the parsed model once into the plain
 * structure-of-arrays `EdenGpuModel` below (engine units of
 * eden/NeuroML.cpp:307-400: us, mV, nA, pF, uS, Mohm, um) and then advances
 * the network any number of steps per call.
 *
 * All entry points return 0 on success and a negative EDEN_GPU_E* code on
 * failure; `edenGpuLastError` gives the message.  Nothing here calls exit(),
 * abort() or traps; device-side faults (a bounded wait that ran out, a
 * non-finite recorded value) are reported through the same codes after the
 * call that saw them.
 */
#ifndef EDEN_GPU_H
#define EDEN_GPU_H

#ifndef __CUDACC_RTC__
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define EDEN_GPU_ABI_VERSION 12

enum {
    EDEN_GPU_OK = 0,
    EDEN_GPU_E_INVALID = -1,   /* malformed model or argument */
    EDEN_GPU_E_CUDA = -2,      /* a CUDA runtime call failed */
    EDEN_GPU_E_NOMEM = -3,     /* device allocation refused */
    EDEN_GPU_E_NONFINITE = -4, /* NaN/Inf in a recorded value */
    EDEN_GPU_E_RANGE = -5,     /* record buffer too small / index out of range */
    EDEN_GPU_E_NODEVICE = -6   /* no CUDA device visible */
};

/* Gate rate forms of ionChannelHH/gateHHrates (eden/Eden.cpp:5164-5181). */
enum {
    EDEN_RATE_EXP = 0,        /* r * exp((V - mid) / s)                     */
    EDEN_RATE_EXPLINEAR = 1,  /* r * x / (1 - exp(-x)), x = (V - mid) / s; r at V == mid */
    EDEN_RATE_SIGMOID = 2,    /* r / (1 + exp((mid - V) / s))               */
    EDEN_RATE_FIXED = 3       /* r (fixedTimeCourse: tau, us)               */
};

/* Gate kinds (eden/NeuroML.cpp:4172-4177; dynamics eden/Eden.cpp:5290-5375):
 * each derives tau and inf from the forward/reverse rates (tau = 1/(a+b),
 * inf = a/(a+b)) unless it has its own timeCourse / steadyState form. */
enum {
    EDEN_GATE_RATES = 0,        /* gateHHrates: forward, reverse            */
    EDEN_GATE_TAUINF = 1,       /* gateHHtauInf: timeCourse, steadyState    */
    EDEN_GATE_RATESTAU = 2,     /* gateHHratesTau: rates, timeCourse        */
    EDEN_GATE_RATESINF = 3,     /* gateHHratesInf: rates, steadyState       */
    EDEN_GATE_RATESTAUINF = 4,  /* gateHHratesTauInf: all four              */
    EDEN_GATE_INSTANTANEOUS = 5,/* gateHHInstantaneous: the steady state at
                                   the step's own V, no state of its own     */
    EDEN_GATE_KINDS = 6
};

#define EDEN_MAX_GATES 4

/* Point-neuron kinds (LEMS_CoreComponents.inc.xml: izhikevich2007Cell
 * 1140-1187, iafTauCell 957-983, iafTauRefCell 985-1021, iafCell 1023-1056,
 * iafRefCell 1058-1095, adExIaFCell 1189-1240). */
enum {
    EDEN_POINT_IZH2007 = 0,
    EDEN_POINT_IAF_TAU = 1,
    EDEN_POINT_IAF_TAU_REF = 2,
    EDEN_POINT_IAF = 3,
    EDEN_POINT_IAF_REF = 4,
    EDEN_POINT_ADEX = 5,
    EDEN_POINT_IZH_DL = 6,      /* izhikevichCell (LEMS_CoreComponents.inc.xml izhikevichCell):
                                   v0, thresh (mV), a, b, c, d (dimensionless); its input
                                   current is dimensionless (the *GeneratorDL inputs) */
    EDEN_POINT_FN = 7,          /* fitzHughNagumoCell: I (dimensionless); V, W dimensionless,
                                   no input current, no spikes */
    EDEN_POINT_KINDS = 8
};
#define EDEN_POINT_PARAMS 16

/* Waveform current inputs (LEMS_CoreComponents.inc.xml: sineGenerator
 * 430-458, rampGenerator 489-521). Parameters of input k at
 * wave_params[EDEN_WAVE_PARAMS * k + j]: j = 0 delay (us), 1 duration (us),
 * then for a sine 2 amplitude (nA), 3 period (us), 4 phase (rad); for a ramp
 * 2 startAmplitude, 3 finishAmplitude, 4 baselineAmplitude (nA). */
enum {
    EDEN_WAVE_SINE = 0,
    EDEN_WAVE_RAMP = 1,
    EDEN_WAVE_SHAPES = 2
};
#define EDEN_WAVE_PARAMS 5

/* Voltage clamps (LEMS_CoreComponents.inc.xml: voltageClamp 555-586,
 * voltageClampTriple 588-620). Parameters of clamp k at
 * clamp_params[EDEN_CLAMP_PARAMS * k + j]: 0 delay (us), 1 duration (us),
 * target potential (mV) 2 before the delay, 3 from the delay to delay +
 * duration, 4 after that (NaN: no current in that phase), 5 series
 * resistance (MOhm). */
#define EDEN_CLAMP_PARAMS 6

/* One ionChannelHH type: up to EDEN_MAX_GATES gateHHrates, each contributing
 * q^instances to the open fraction (eden/Eden.cpp:5678-5717). Rates in 1/us. */
typedef struct EdenGpuChannelType {
    int32_t n_gates;
    int32_t gate_instances[EDEN_MAX_GATES];
    int32_t fwd_kind[EDEN_MAX_GATES];
    float fwd_rate[EDEN_MAX_GATES], fwd_mid[EDEN_MAX_GATES], fwd_scale[EDEN_MAX_GATES];
    int32_t rev_kind[EDEN_MAX_GATES];
    float rev_rate[EDEN_MAX_GATES], rev_mid[EDEN_MAX_GATES], rev_scale[EDEN_MAX_GATES];
    float q10[EDEN_MAX_GATES];      /* rate scale of each gate (q10Settings at the network's temperature) */
    int32_t gate_kind[EDEN_MAX_GATES];                                   /* EDEN_GATE_* */
    int32_t tau_kind[EDEN_MAX_GATES];                                    /* timeCourse form */
    float tau_rate[EDEN_MAX_GATES], tau_mid[EDEN_MAX_GATES], tau_scale[EDEN_MAX_GATES];
    int32_t inf_kind[EDEN_MAX_GATES];                                    /* steadyState form (rate dimensionless) */
    float inf_rate[EDEN_MAX_GATES], inf_mid[EDEN_MAX_GATES], inf_scale[EDEN_MAX_GATES];
} EdenGpuChannelType;

enum { EDEN_SYN_EXPONE = 0, EDEN_SYN_EXPTWO = 1, EDEN_SYN_ALPHA = 2, EDEN_SYN_ALPHA_CURRENT = 3,
       EDEN_SYN_EXPONE_CURRENT = 4, EDEN_SYN_BLOCKING_PLASTIC = 5 };
enum { EDEN_CABLE_BWD_EULER = 0, EDEN_CABLE_FWD_EULER = 1 };
#define EDEN_GRADED_PARAMS 5

/* expOneSynapse (native, eden/Eden.cpp:3424-3466), expTwoSynapse,
 * alphaSynapse or alphaCurrentSynapse (LEMS, LEMS_CoreComponents.inc.xml:
 * 85-180).  gbase uS, erev mV, taus us.  `waveform_factor` is expTwo's
 * derived 1/(-exp(-tp/tr)+exp(-tp/td)) and `weight_prop` its LEMS `weight`
 * property (default 1).  The alpha kinds have one time constant, in
 * tau_decay; an alphaCurrentSynapse carries its ibase (nA) in gbase and
 * contributes current only (erev unused).  EDEN_SYN_EXPONE_CURRENT is
 * PyNN's expCurrSynapse (LEMS_CoreComponents.inc.xml:1858-1877): expOne's
 * state, jumping by gbase (nA) and decaying with tau_decay, taken as a
 * current.  PyNN's expCondSynapse, alphaCondSynapse and alphaCurrSynapse
 * are EDEN_SYN_EXPONE, EDEN_SYN_ALPHA and EDEN_SYN_ALPHA_CURRENT with
 * gbase 1 (uS or nA), and an expThreeSynapse is two EDEN_SYN_EXPTWO types
 * on the same connection. */
typedef struct EdenGpuSynapseType {
    int32_t kind;
    float gbase, erev, tau_decay, tau_rise, waveform_factor, weight_prop;
    /* EDEN_SYN_BLOCKING_PLASTIC (blockingPlasticSynapse,
     * LEMS_CoreComponents.inc.xml:231-352): expTwo's A and B with each
     * event's jump scaled by the plasticity factor R U before the event;
     * tsodyksMarkram(DepFac)Mechanism: R' = (1 - R) / tau_rec,
     * U' = (release_prob - U) / tau_fac (tau_fac 0: U = release_prob, the
     * depression-only mechanism), on an event R = R (1 - U),
     * U = U + release_prob (1 - U); R = 1, U = release_prob at start
     * (tau_rec 0: no plasticity, factor 1).  voltageConcDepBlockMechanism:
     * g = B(V) gbase (B - A) with B(V) = 1 / (1 + block_ratio exp(-V /
     * block_volt)), block_ratio = blockConcentration / scalingConc
     * (block_volt 0: no block).  Connections only; such a model runs the
     * per-step kernels. */
    float release_prob, tau_rec, tau_fac, block_ratio, block_volt;
} EdenGpuSynapseType;

/*
 * The lowered network.  "Targets" are the places a membrane potential lives:
 * targets [0, n_comp) are the compartments of physical cells (cell by cell,
 * each cell's compartments in the reference's compartment order), targets
 * [n_comp, n_comp + n_izh) are point neurons (izhikevich2007Cell, iaf*Cell,
 * adExIaFCell).
 * Every array is host memory, read during edenGpuCreate only.
 */
typedef struct EdenGpuModel {
    int32_t abi_version;      /* EDEN_GPU_ABI_VERSION */
    float dt;                 /* us */
    int64_t seed;             /* simulation RNG seed */

    /* physical cells and their compartments */
    int32_t n_phys;
    const int32_t *phys_comp_off;   /* [n_phys + 1] */
    int32_t n_comp;
    const int32_t *comp_parent;     /* [n_comp] parent within the cell, -1 at the root */
    const float *comp_c;            /* [n_comp] capacitance, pF */
    const float *comp_r_axial;      /* [n_comp] axial resistance to the parent, Mohm (root: unused) */
    const float *comp_area;         /* [n_comp] membrane area, um2 */
    const float *comp_inv_rc;       /* [n_comp] sum over neighbours of 1/(R*C), 1/us */
    const float *comp_v0;           /* [n_comp] initial V, mV */

    /* channel instances (channelDensity on a compartment), grouped by compartment */
    int32_t n_chan_types;
    const EdenGpuChannelType *chan_types;
    const int32_t *comp_chan_off;   /* [n_comp + 1] */
    const int32_t *chan_type;       /* [n_chan] */
    const float *chan_gbase;        /* [n_chan] conductivity, mS/cm2 */
    const float *chan_erev;         /* [n_chan] mV */

    /* point neurons (the reference's LEMS-defined artificial cells,
     * eden/Eden.cpp:6821-6914), one kind each (izh_kind, EDEN_POINT_*),
     * parameters in engine units at izh_params[EDEN_POINT_PARAMS * i + k]:
     *   IZH2007      C pF, v0 mV, k nS/mV, vr, vt, vpeak mV, a 1/us, b uS, c mV, d nA
     *   IAF_TAU      leakReversal mV, tau us, thresh, reset mV
     *   IAF_TAU_REF  leakReversal mV, tau us, thresh, reset mV, refract us
     *   IAF          C pF, leakConductance uS, leakReversal, thresh, reset mV
     *   IAF_REF      C pF, leakConductance uS, leakReversal, thresh, reset mV, refract us
     *   ADEX         C pF, gL uS, EL, VT, thresh, reset, delT mV, tauw us, refract us,
     *                a uS, b nA */
    int32_t n_izh;
    const float *izh_params;

    /* spike sources: one per cell (gid order); `src_target` is the target
     * whose threshold crossing (physical: V < thr < V_next, eden/Eden.cpp:6248)
     * or izhikevich v > vpeak (LEMS OnCondition) emits the spike */
    int32_t n_src;
    const int32_t *src_target;      /* [n_src] */
    const float *src_threshold;     /* [n_src] mV, physical sources only */
    const int32_t *src_cell_seed;   /* [n_src] reverse_bits(seed) ^ gid (eden/Eden.cpp:7679-7691) */

    /* synapse types and connection synapses (connectionWD instances) */
    int32_t n_syn_types;
    const EdenGpuSynapseType *syn_types;
    int64_t n_syn;
    const int32_t *syn_target;      /* [n_syn] */
    const int32_t *syn_type;        /* [n_syn] */
    const int32_t *syn_src;         /* [n_syn] presynaptic source */
    const float *syn_weight;        /* [n_syn] connection weight */
    const float *syn_delay;         /* [n_syn] us */

    /* poissonFiringSynapse inputs, each with its own synapse instance */
    int64_t n_pois;
    const int32_t *pois_target;
    const int32_t *pois_type;       /* synapse type it drives */
    const float *pois_rate;         /* 1/us */
    const float *pois_weight;
    const int32_t *pois_src;        /* cell (spike source index) whose RNG seed it uses */
    const int32_t *pois_instance;   /* instance number in the reference's per-cell input table */

    /* pulseGenerator inputs */
    int64_t n_pulse;
    const int32_t *pulse_target;
    const float *pulse_start, *pulse_duration, *pulse_amplitude, *pulse_weight; /* us, us, nA, - */

    /* per-target input order: within each target the reference sums channel,
     * then input (pulse, Poisson), then synapse currents (eden/Eden.cpp:6057-6060) */

    /* spikes of sources with no target (src_target -1: spikeArray and
     * spikeGenerator populations, eden/Eden.cpp:6738-6790), known in advance:
     * source and the step at which each is logged (the step after the one
     * that emits it), sorted by step; delivered through the fan-out like a
     * cell's spikes */
    int64_t n_ext;
    const int32_t *ext_src;
    const int64_t *ext_step;

    const int32_t *izh_kind;        /* [n_izh] EDEN_POINT_* of each point neuron */

    /* timedSynapticInput inputs, each with its own synapse instance, which
     * fires in the listed steps (the first step whose t + dt exceeds a spike
     * time, eden/Eden.cpp:3759-3790, 3859-3871; increasing, >= 1) */
    int64_t n_timed;
    const int32_t *timed_target;
    const int32_t *timed_type;      /* synapse type it drives */
    const float *timed_weight;
    const int64_t *timed_off;       /* [n_timed + 1] into timed_step */
    const int64_t *timed_step;

    /* sineGenerator / rampGenerator inputs: the current at a step is
     * wave_weight * f(t), t the step's time, as the reference's LEMS code
     * exposes the value its OnConditions assign in the same step
     * (eden/Eden.cpp:3107-3133, 2832-2994) */
    int64_t n_wave;
    const int32_t *wave_target;
    const int32_t *wave_shape;      /* EDEN_WAVE_* */
    const float *wave_params;       /* [n_wave * EDEN_WAVE_PARAMS] */
    const float *wave_weight;

    /* per Poisson input, the random-call id of its first draw (its second
     * is the next): the random calls of the compartments before it in its
     * cell type plus two per Poisson component before it on its own
     * compartment (eden/Eden.cpp:6540, 2450-2458); NULL for all 0 */
    const int32_t *pois_rng_base;

    /* voltage clamps: current clamp_weight * (target - V) / R, V the
     * compartment's potential at the start of the step, the target of the
     * step's phase (the OnConditions' last assignment at its time) */
    int64_t n_clamp;
    const int32_t *clamp_target;
    const float *clamp_params;      /* [n_clamp * EDEN_CLAMP_PARAMS] */
    const float *clamp_weight;

    /* gap junctions (gapJunction on electricalConnection(Instance)(W)): one
     * entry per end, each on a physical compartment, taking
     * weight * conductance * (V_peer - V) as synaptic current with the
     * peer's potential at the start of the step and no conductance term
     * (eden/Eden.cpp:3407-3422, 3689-3704; both ends 9233-9251).  Cells
     * coupled this way influence each other within a step, so a model with
     * gap junctions runs one-step windows. */
    int64_t n_gap;
    const int32_t *gap_target;      /* compartment the end sits on */
    const int32_t *gap_peer;        /* compartment at the other end */
    const float *gap_conductance;   /* uS */
    const float *gap_weight;

    /* cable solver of the physical cells (the reference's command-line
     * `cable_solver`, eden/Eden.cpp:10485-10500): EDEN_CABLE_BWD_EULER, its
     * default, the backward-Euler Hines solve; or EDEN_CABLE_FWD_EULER, the
     * explicit update V_next = V + dt (I + I_axial) / C with
     * I_axial = sum of (V_adj - V) / R over the compartment's neighbours
     * in ascending compartment order (parent, then children), from the
     * potentials at the start of the step (4969-4990, 6092-6094).  A
     * forward-Euler model runs the per-step kernels in either mode. */
    int32_t cable_solver;

    /* gradedSynapse ends (continuous connections, LEMS_CoreComponents.inc.xml:
     * 38-80; instantiated on each end like gap junctions, eden/Eden.cpp:
     * 9254-9270): on compartment `graded_target`, with the potential of
     * `graded_peer` at the step's start as vpeer,
     *   inf = 1 / (1 + exp((Vth - vpeer) / delta)),  tau = (1 - inf) / k,
     *   i = weight * conductance * s * (erev - V)   (current only),
     *   s' = (inf - s) / tau while 1 - inf > 1e-4, else s = inf; s = 0 at start.
     * graded_params per end: conductance (uS), delta (mV), k (1/us), Vth
     * (mV), erev (mV).  A linearGradedSynapse end is a gap-junction end
     * above; a silentSynapse end is nothing.  Like gap junctions they run
     * one-step windows. */
    int64_t n_graded;
    const int32_t *graded_target;
    const int32_t *graded_peer;
    const float *graded_params;     /* [n_graded * EDEN_GRADED_PARAMS] */
    const float *graded_weight;
} EdenGpuModel;

/* Execution options. */
enum { EDEN_MODE_PLAIN = 0, EDEN_MODE_BATCHED = 1 };
typedef struct EdenGpuOptions {
    int32_t mode;             /* EDEN_MODE_PLAIN: one set of launches per step;
                                 EDEN_MODE_BATCHED: multi-step windows, graph-captured */
    int32_t device;           /* CUDA device ordinal */
    int32_t steps_per_launch; /* batched window length; 0 = autotune (bounded by the minimum delay) */
    int32_t cells_per_block;  /* 0 = autotune */
    int32_t record_capacity_steps; /* trace samples buffered on the device between fetches */
    int32_t spike_capacity;   /* spike events buffered on the device between fetches */
    int32_t n_trace;          /* recorded columns */
    const int32_t *trace_target; /* per column: a target (its membrane potential), or -2 - g for
                                    the state of gate g of the physical compartments' channel
                                    instances, numbered instance by instance in comp_chan_off
                                    order and within one in its type's gate order (the gate
                                    paths of an OutputColumn, eden/NeuroML.cpp:8140-8183) */
    int32_t kernel_timing;    /* 1: bracket every kernel launch with CUDA events (no graph
                                 replay) and accumulate per-kernel device time */
    int32_t codegen;          /* batched mode: 0 = compile the windowed kernels for the
                                 model's channel sets with NVRTC when available (else use
                                 the built-in ones), 1 = require it, -1 = built-in kernels */
    int32_t max_cell_blocks;  /* batched mode: most blocks of one windowed cell-kernel launch
                                 (0 = 32 per SM); with fewer blocks than CTAs each block runs
                                 several CTAs in turn */
    int32_t segments_per_warp;  /* most compartments of one warp's forest of cells (0 = sized
                                   to the network, at most 768; at most 1023); a larger cell
                                   gets a warp of its own */
    int32_t segments_per_depth; /* most compartments of a forest at one depth (0 = 64) */
    int32_t reserved[3];
} EdenGpuOptions;

/* Kernels whose device time kernel_timing accumulates. */
enum {
    EDEN_KERNEL_INPUTS = 0,   /* synapse / Poisson / pulse input blocks */
    EDEN_KERNEL_CELLS = 1,    /* windowed cell kernel (batched mode) */
    EDEN_KERNEL_TARGETS = 2,  /* per-step target kernel (plain mode) */
    EDEN_KERNEL_HINES = 3,    /* per-step cable solve (plain mode) */
    EDEN_KERNEL_DELIVER = 4,  /* spike fan-out */
    EDEN_KERNEL_KINDS = 5
};

/* Records produced since the previous fetch, in step order. */
typedef struct EdenGpuRecords {
    /* caller-provided host buffers and their capacities */
    float *trace;             /* [trace_capacity * n_trace], sample-major */
    int64_t *trace_step;      /* [trace_capacity] step index of each sample */
    int64_t trace_capacity;
    int32_t *spike_src;       /* [spike_capacity] */
    int64_t *spike_step;      /* [spike_capacity] step at which the spike is logged */
    int64_t spike_capacity;
    /* filled in */
    int64_t n_trace_samples;
    int64_t n_spikes;
    /* optional (NULL: not copied), [spike_capacity]: each spike's
     * threshold-crossing time in us, interpolated in double between the
     * potential at the start and at the end of the step that crossed
     * (NaN for point neurons and sources with no membrane).  A diagnostic
     * beside spike_step, which stays the reference's quantised time
     * (eden/Eden.cpp:6247-6252). */
    double *spike_time_us;
} EdenGpuRecords;

typedef struct EdenGpuCtx EdenGpuCtx;

/* (the entry points are host functions; the types above are also compiled
 * into the library's run-time generated kernels, which see no declarations) */
#ifndef __CUDACC_RTC__

/* Build a context: validate the model, upload it to device memory in the
 * GPU layout, build the spike fan-out table.  Replaces the reference's
 * GenerateModel() output tables (eden/Eden.cpp:677, RawTables 446-532)
 * and the now/next buffer allocation (11095-11150). */
int edenGpuCreate(const EdenGpuModel *model, const EdenGpuOptions *opt, EdenGpuCtx **out);

/* Advance `n_steps` steps starting at step index `first_step`.  Step indices
 * follow the reference loop (eden/Eden.cpp:11488-11510): steps <= 0 are the
 * initialisation passes at t = 0, step k >= 1 runs at t = (k - 1) * dt.
 * Records the state at the start of every non-initialisation step (the
 * reference's output phase, 11555-11635). */
int edenGpuRun(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps);

/* edenGpuRun for callers that cannot allocate while the simulation runs (no
 * counterpart in the reference, whose loop runs on the host).  edenGpuRun may
 * allocate during a call -- it grows its window table when a call spans more
 * windows than the table holds, and its first batched call instantiates a
 * CUDA graph -- which a caller holding a fixed device-memory budget, or one
 * that cannot let cudaMalloc/cudaFree synchronise the device mid-run, must
 * avoid.  This entry point runs the same kernels in the same order and
 * allocates nothing: the input scratch lives in a static device array of
 * 16 MiB (models of at most 131072 input chunks; a chunk is up to 128
 * inputs of one type on one compartment; larger models get EDEN_GPU_E_RANGE), window arguments in a static device table, and the
 * launches are direct (no graph, no kernel timing).  Results equal
 * edenGpuRun's; the two may be interleaved on one context.
 * The first call on a context performs a one-time set-up (looking up the
 * static arrays' device addresses with the context's device current);
 * n_steps = 0 does only that, and it should come before any stream capture
 * starts.  The static arrays belong to the library's module, so every device
 * that loads the library's kernels holds their 16 MiB until the process
 * exits, whether or not this entry point is used.  They are shared by all
 * contexts on a device and keep the last call's contents: calls that
 * overlap in time on one device race on them, so serialise them.
 * A run that fails before issuing any kernel leaves the context as it was;
 * one that fails after (edenGpuRun too) leaves it refusing further runs. */
int edenGpuRunStaticScratch(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps);

/* Copy records accumulated since the last fetch into caller buffers. */
int edenGpuFetchRecords(EdenGpuCtx *ctx, EdenGpuRecords *rec);

/* Read / write membrane potentials of all targets (n_comp + n_izh floats). */
int edenGpuReadV(EdenGpuCtx *ctx, float *v_host, int64_t n);
int edenGpuWriteV(EdenGpuCtx *ctx, const float *v_host, int64_t n);

/* Per-synapse pending spike times (us) and synapse state, for routing checks. */
int edenGpuReadSynapses(EdenGpuCtx *ctx, float *pending_us, float *state_a, float *state_b, int64_t n);

/* The number of physical cells whose cable solve runs in double precision.
 * A row of the backward-Euler cable matrix (eden/Eden.cpp:6114-6225) is
 * diagonally dominant whenever its compartment's membrane conductance is
 * not negative; edenGpuCreate flags every cell that can get a negative one
 * (a negative channel density, synaptic gbase, expTwo jump or weight on any
 * of its compartments) and eliminates its matrix in double precision, the
 * state staying single precision.  (No reference counterpart: the reference
 * solves every cell in single precision.) */
int edenGpuFp64Cells(EdenGpuCtx *ctx, int64_t *n_cells);

/* Device time of the last edenGpuRun in milliseconds and the number of
 * kernel launches it issued. */
int edenGpuLastRunStats(EdenGpuCtx *ctx, double *device_ms, int64_t *launches);

/* Per-kernel device time accumulated since creation when kernel_timing is
 * set (the reference's only timing is its Config/Setup/Run wall-clock line,
 * eden/Eden.cpp:11951; this is the GPU-side breakdown of Run). */
int edenGpuKernelStats(EdenGpuCtx *ctx, int32_t kind, double *total_ms, int64_t *launches);

/* The CUDA source compiled at creation for this model's windowed kernels
 * (batched mode with codegen >= 0: the library's kernels plus one routine
 * per channel set, the counterpart of the C the reference generates per cell
 * type, eden/Eden.cpp:7017-7180).  Copies at most cap - 1 bytes and a NUL
 * into buf when buf is not null; returns the source length, 0 when the
 * built-in kernels run, or a negative error code. */
int64_t edenGpuGeneratedSource(EdenGpuCtx *ctx, char *buf, int64_t cap);

const char *edenGpuLastError(EdenGpuCtx *ctx);
void edenGpuDestroy(EdenGpuCtx *ctx);
int edenGpuAbiVersion(void);

/*
 * Gradients (no counterpart in the reference, which has no gradient path).
 *
 * For models of independent physical cells -- HH channels
 * (ionChannelHH/gateHHrates), pulse inputs, and synaptic drive whose events
 * are fixed in advance: timedSynapticInput inputs and connection synapses
 * from spike sources without a membrane (spike lists, generators, event-set
 * readers); no Poisson inputs, no point neurons, no synapse from a cell that
 * spikes -- the library runs the same step as edenGpuRun's plain
 * path (gates eden/Eden.cpp:5126-5259, channel currents 5805-5898, synapses
 * 3424-3466 and LEMS_CoreComponents.inc.xml:145-180 with the weight product
 * of 3708-3710, V pre-update 6057-6107, Hines solve 6114-6225) with chosen
 * channel conductivities, cell axial resistivities and synaptic weights
 * taken from a parameter vector,
 * records the membrane potential of chosen compartments at the start of
 * steps 1..n_steps, and returns the gradient of any scalar function of that
 * trace with respect to the parameters, given the function's gradient with
 * respect to the trace: the discrete adjoint of the step, run backward in
 * time over segments recomputed from forward states stored every
 * `checkpoint_every` steps.
 *
 * Pointers to parameters, traces and gradients may be host or device
 * memory.  Calls are synchronous.
 */
typedef struct EdenGpuGradSpec {
    int32_t n_params;
    const int32_t *chan_param;     /* [n_chan] parameter that is the channel's conductivity
                                      (mS/cm2), or -1 to keep chan_gbase; may be null */
    const int32_t *cell_ra_param;  /* [n_phys] parameter that is the cell's axial resistivity
                                      (ohm cm), or -1; may be null */
    const float *cell_ra;          /* [n_phys] the resistivity (ohm cm) that comp_r_axial and
                                      comp_inv_rc were computed with; needed with cell_ra_param */
    int32_t n_rec;
    const int32_t *rec_comp;       /* [n_rec] compartments recorded as trace columns */
    int64_t n_steps;               /* trace rows: steps 1..n_steps */
    int32_t checkpoint_every;      /* steps per recomputed segment; 0 = 100 */
    int32_t device;
    const int32_t *syn_param;      /* [n_syn] parameter that is the connection's weight, or -1 to
                                      keep syn_weight; may be null */
    const int32_t *timed_param;    /* [n_timed] parameter that is the input's weight, or -1 to keep
                                      timed_weight; may be null */
    int32_t reserved[4];
} EdenGpuGradSpec;

typedef struct EdenGpuGrad EdenGpuGrad;

/* Validate and upload; *out is set even on failure (read the message with
 * edenGpuGradLastError, then destroy it). */
int edenGpuGradCreate(const EdenGpuModel *model, const EdenGpuGradSpec *spec, EdenGpuGrad **out);

/* Run the initialisation passes and steps 1..n_steps with `params`
 * ([n_params]); write the trace ([n_steps * n_rec], step-major) and keep the
 * checkpoints for the next edenGpuGradBackward. */
int edenGpuGradForward(EdenGpuGrad *g, const float *params, float *trace);

/* Gradient ([n_params]) of a scalar function of the last forward's trace,
 * given that function's gradient with respect to the trace
 * ([n_steps * n_rec]).  Parameters that no channel or cell uses get 0. */
int edenGpuGradBackward(EdenGpuGrad *g, const float *trace_grad, float *param_grad);

/* Device time in milliseconds of the last forward and backward calls. */
int edenGpuGradTiming(EdenGpuGrad *g, double *forward_ms, double *backward_ms);

const char *edenGpuGradLastError(EdenGpuGrad *g);
void edenGpuGradDestroy(EdenGpuGrad *g);
#endif /* __CUDACC_RTC__ */

#ifdef __cplusplus
}
#endif
#endif
