"""Lower a NetworkSpec into the engine-unit arrays of `EdenGpuModel`.

This mirrors what the reference's GenerateModel() computes for the
mechanisms of this path (eden/Eden.cpp:677-10378), with single precision
where the reference stores `Real` (float):

* units: quantities are converted as ScaleEntry::ConvertTo does
  (eden/NeuroML.h:530-532): value * 10^(pow_from - pow_native) in double,
  then stored as float.  Engine units are us, mV, nA, pF, uS, Mohm, um
  (eden/NeuroML.cpp:307-400);
* compartments: one per segment, in segment order; area of a cylinder
  pi*d*L, of a zero-length segment pi*d^2 (GeomHelp::Area,
  eden/Eden.cpp:242-252); capacitance = Cm * area
  (eden/Eden.cpp:4222-4226); axial resistance between a compartment and its
  parent = proximal half of the child + distal half of the parent, each
  Ra*(4/pi)*len/(d_from*d_to) (eden/Eden.cpp:4228-4241, 4256-4308,
  4340-4347); the fixed diagonal sum of 1/(R*C) over neighbours
  (eden/Eden.cpp:4488-4501);
* per-cell RNG seed reverse_bits(seed) ^ gid (eden/Eden.cpp:7672-7691);
* expTwoSynapse's derived peakTime / waveformFactor evaluated in float
  the way the generated code does (LEMS_CoreComponents.inc.xml:152-153).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from .network import (SPIKE_SOURCE_TYPES, AdExCell, EventSetReaderCell, FitzHughNagumoCell, IafCell,
                      Izhikevich2007Cell, IzhikevichCell,
                      NetworkSpec,
                      PhysicalCell, SpikeArrayCell, SpikeGeneratorPoissonCell, SpikeGeneratorRandomCell,
                      WAVE_RAMP, WAVE_SINE,
                      SYN_EXPTWO, SYN_ALPHA_CURRENT, SYN_EXPONE_CURRENT, SYN_EXPTHREE, SYN_BLOCKING_PLASTIC, SynapseType)

F32 = np.float32
MAX_GATES = 4


def _to_f32(x) -> np.float32:
    return F32(float(x))


def ms_to_us(x):
    return np.asarray(x, dtype=np.float64) * 1000.0


def reverse_bits32(x: int) -> int:
    x &= 0xFFFFFFFF
    x = ((x & 0xFFFF0000) >> 16) | ((x & 0x0000FFFF) << 16)
    x = ((x & 0xFF00FF00) >> 8) | ((x & 0x00FF00FF) << 8)
    x = ((x & 0xF0F0F0F0) >> 4) | ((x & 0x0F0F0F0F) << 4)
    x = ((x & 0xCCCCCCCC) >> 2) | ((x & 0x33333333) << 2)
    x = ((x & 0xAAAAAAAA) >> 1) | ((x & 0x55555555) << 1)
    return x & 0xFFFFFFFF


def cell_seeds(seed: int, n: int) -> np.ndarray:
    r = reverse_bits32(int(seed) & 0xFFFFFFFF)
    s = (np.uint32(r) ^ np.arange(n, dtype=np.uint32)).astype(np.uint32)
    return s.view(np.int32)


def exptwo_waveform_factor(tau_rise_us: float, tau_decay_us: float) -> np.float32:
    """peakTime and waveformFactor in float, as the generated kernel
    evaluates LEMS_CoreComponents.inc.xml:152-153."""
    tr, td = F32(tau_rise_us), F32(tau_decay_us)
    with np.errstate(all="ignore"):
        tp = F32(F32(F32(np.log(F32(td / tr))) * F32(F32(tr * td) * F32(1e-12))) / F32(td - tr)) * F32(1e12)
        tp = F32(tp)
        wf = F32(1.0) / F32(-np.exp(F32(-tp / tr)) + np.exp(F32(-tp / td)))
    return F32(wf)


# ---------------------------------------------------------------------------
@dataclass
class LoweredModel:
    dt: np.float32
    seed: int
    n_steps: int
    # physical
    phys_comp_off: np.ndarray
    comp_parent: np.ndarray
    comp_c: np.ndarray
    comp_r_axial: np.ndarray
    comp_area: np.ndarray
    comp_inv_rc: np.ndarray
    comp_v0: np.ndarray
    chan_types: np.ndarray        # structured, see CHAN_DTYPE
    comp_chan_off: np.ndarray
    chan_type: np.ndarray
    chan_gbase: np.ndarray
    chan_erev: np.ndarray
    # point neurons
    izh_params: np.ndarray        # [n_izh, POINT_PARAMS] point-neuron parameters, engine units
    # spike sources (one per gid)
    src_target: np.ndarray
    src_threshold: np.ndarray
    src_cell_seed: np.ndarray
    # synapses
    syn_types: np.ndarray         # structured, see SYN_DTYPE
    syn_target: np.ndarray
    syn_type: np.ndarray
    syn_src: np.ndarray
    syn_weight: np.ndarray
    syn_delay: np.ndarray
    # poisson
    pois_target: np.ndarray
    pois_type: np.ndarray
    pois_rate: np.ndarray
    pois_weight: np.ndarray
    pois_src: np.ndarray
    pois_instance: np.ndarray
    # pulses
    pulse_target: np.ndarray
    pulse_start: np.ndarray
    pulse_duration: np.ndarray
    pulse_amplitude: np.ndarray
    pulse_weight: np.ndarray
    # recording
    trace_target: np.ndarray
    event_src: np.ndarray         # spike source recorded by each EventSelection
    # bookkeeping
    gid_target_base: np.ndarray = field(default=None)  # first target of each gid
    chan_density: np.ndarray = field(default=None)     # channel -> index of its channelDensity in the cell type
    # spikes of the sources with no target, (source, logging step), in step order
    ext_src: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    ext_step: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    izh_kind: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))  # POINT_* per point neuron
    # timedSynapticInput: target, synapse type, weight, and the steps each fires in
    timed_target: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    timed_type: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    timed_weight: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    timed_off: np.ndarray = field(default_factory=lambda: np.zeros(1, np.int64))
    timed_step: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    phys_ra: np.ndarray = field(default=None)          # physical cell -> axial resistivity, ohm*cm
    # sineGenerator / rampGenerator: target, WAVE_* shape, [n, WAVE_PARAMS] parameters (engine units), weight
    wave_target: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    wave_shape: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    wave_params: np.ndarray = field(default_factory=lambda: np.zeros((0, 5), np.float32))
    wave_weight: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    # per Poisson input, the random-call id of its first draw
    pois_rng_base: np.ndarray = field(default=None)
    # voltage clamps: target, [n, CLAMP_PARAMS] parameters (engine units), weight
    clamp_target: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    clamp_params: np.ndarray = field(default_factory=lambda: np.zeros((0, 6), np.float32))
    clamp_weight: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    # gap junctions: one entry per end (the compartment it sits on, the peer
    # compartment, conductance uS, weight)
    gap_target: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    gap_peer: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    gap_conductance: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    gap_weight: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    # cable solver of the physical cells: CABLE_BWD_EULER or CABLE_FWD_EULER
    cable_solver: int = 0
    # gradedSynapse ends: the compartment, the peer compartment, [n, 5]
    # (conductance uS, delta mV, k 1/us, Vth mV, erev mV), weight
    graded_target: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    graded_peer: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    graded_params: np.ndarray = field(default_factory=lambda: np.zeros((0, 5), np.float32))
    graded_weight: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))

    @property
    def n_comp(self) -> int:
        return int(len(self.comp_c))

    @property
    def n_izh(self) -> int:
        return int(len(self.izh_params))

    @property
    def n_target(self) -> int:
        return self.n_comp + self.n_izh

    @property
    def n_phys(self) -> int:
        return int(len(self.phys_comp_off) - 1)


CHAN_DTYPE = np.dtype([
    ("n_gates", np.int32), ("gate_instances", np.int32, MAX_GATES),
    ("fwd_kind", np.int32, MAX_GATES), ("fwd_rate", np.float32, MAX_GATES),
    ("fwd_mid", np.float32, MAX_GATES), ("fwd_scale", np.float32, MAX_GATES),
    ("rev_kind", np.int32, MAX_GATES), ("rev_rate", np.float32, MAX_GATES),
    ("rev_mid", np.float32, MAX_GATES), ("rev_scale", np.float32, MAX_GATES),
    ("q10", np.float32, MAX_GATES),
    ("gate_kind", np.int32, MAX_GATES),
    ("tau_kind", np.int32, MAX_GATES), ("tau_rate", np.float32, MAX_GATES),
    ("tau_mid", np.float32, MAX_GATES), ("tau_scale", np.float32, MAX_GATES),
    ("inf_kind", np.int32, MAX_GATES), ("inf_rate", np.float32, MAX_GATES),
    ("inf_mid", np.float32, MAX_GATES), ("inf_scale", np.float32, MAX_GATES),
], align=True)

SYN_DTYPE = np.dtype([
    ("kind", np.int32), ("gbase", np.float32), ("erev", np.float32),
    ("tau_decay", np.float32), ("tau_rise", np.float32),
    ("waveform_factor", np.float32), ("weight_prop", np.float32),
    ("release_prob", np.float32), ("tau_rec", np.float32), ("tau_fac", np.float32),
    ("block_ratio", np.float32), ("block_volt", np.float32),
], align=True)


def _cable_geometry(cell: PhysicalCell):
    """Per-compartment C (pF), R to parent (Mohm), area (um2), sum 1/(RC)."""
    n = cell.n_seg
    L = np.asarray(cell.seg_len, np.float64)
    d = np.asarray(cell.seg_diam, np.float64)
    dp = d if cell.seg_dprox is None else np.asarray(cell.seg_dprox, np.float64)
    # floats of the XML coordinates, as the reference parses them; the
    # lateral area of each segment's frustum (eden/Eden.cpp:241-253)
    area = np.where(L == 0, np.pi * d * d,
                    (np.pi / 2.0) * (dp + d) * np.sqrt((dp - d) * (dp - d) / 4.0 + L * L)).astype(F32)
    cm_native = _to_f32(cell.cm)                      # uF/cm2, native
    c = (area.astype(np.float64) * float(cm_native) * 1e-2).astype(F32)
    ra_native = _to_f32(cell.ra * 1e-3)               # ohm*cm -> kohm*cm
    # each half's resistance as a frustum from its end to the midpoint
    # diameter, Ra (4 / pi) length / (d_from d_to) (eden/Eden.cpp:4234-4241,
    # 4304-4305); a zero-length segment as a cylinder as long as it is wide
    half = np.where(L == 0, d / 2.0, L / 2.0)
    dm = np.where(L == 0, d, dp + (d - dp) * 0.5)   # the midpoint's diameter (d for a cylinder)
    dpx = np.where(L == 0, d, dp)
    r_prox = (float(ra_native) * (4.0 / np.pi) * half / (dpx * dm) * 10.0).astype(F32)
    r_dist = (float(ra_native) * (4.0 / np.pi) * half / (dm * d) * 10.0).astype(F32)
    parent = np.asarray(cell.seg_parent, np.int64)
    r_axial = np.full(n, np.nan, dtype=F32)
    inv_rc = np.zeros(n, dtype=F32)
    ci = np.nonzero(parent >= 0)[0]
    if len(ci):
        pi = parent[ci]
        r_axial[ci] = (r_prox[ci] + r_dist[pi]).astype(F32)
        r64 = r_axial[ci].astype(np.float64)
        # edge (i, p) contributes to both ends; a node's own edge comes first,
        # then its children's in increasing order (the order of a loop over i)
        inv_rc[ci] = (1.0 / (r64 * c[ci].astype(np.float64))).astype(F32)
        np.add.at(inv_rc, pi, (1.0 / (r64 * c[pi].astype(np.float64))).astype(F32))
    return c, r_axial, area, inv_rc


# point-neuron kinds and parameter layout (include/eden_gpu.h, EDEN_POINT_*)
POINT_PARAMS = 16
# gate kinds and the fixed rate form (include/eden_gpu.h EDEN_GATE_*, EDEN_RATE_FIXED)
RATE_FIXED = 3
GATE_KINDS = {"rates": 0, "tauInf": 1, "ratesTau": 2, "ratesInf": 3, "ratesTauInf": 4, "instantaneous": 5}


def gate_q10(gate, temperature_degc: float) -> np.float32:
    """A gate's rate scale: 1 without q10Settings, the fixed factor for
    q10Fixed, and q10Factor^((T - experimentalTemp) / 10) for q10ExpTemp
    with both temperatures in kelvin, in single precision as the
    reference's kernel evaluates it (eden/Eden.cpp:5232-5246)."""
    q = gate.q10
    if q is None:
        return F32(1.0)
    if q[0] == "fixed":
        return _to_f32(q[1])
    t = _to_f32(temperature_degc + 273.15)
    tb = _to_f32(q[2] + 273.15)
    return F32(np.power(_to_f32(q[1]), F32(F32(t - tb) / F32(10.0))))


# waveform inputs (include/eden_gpu.h EDEN_WAVE_*)
WAVE_PARAMS = 5
WAVE_SHAPES = {WAVE_SINE: 0, WAVE_RAMP: 1}
POINT_IZH2007, POINT_IAF_TAU, POINT_IAF_TAU_REF, POINT_IAF, POINT_IAF_REF, POINT_ADEX, POINT_IZH_DL, POINT_FN = range(8)
_IAF_KINDS = {"iafTauCell": POINT_IAF_TAU, "iafTauRefCell": POINT_IAF_TAU_REF, "iafCell": POINT_IAF,
              "iafRefCell": POINT_IAF_REF}


def point_params(ct):
    """(kind, parameters in engine units: pF, uS, mV, us, nA) of a point neuron."""
    if isinstance(ct, Izhikevich2007Cell):
        return POINT_IZH2007, [ct.C, ct.v0, ct.k, ct.vr, ct.vt, ct.vpeak, ct.a * 1e-3, ct.b * 1e-3, ct.c, ct.d * 1e-3]
    if isinstance(ct, IafCell):
        kind = _IAF_KINDS[ct.kind]
        if kind in (POINT_IAF_TAU, POINT_IAF_TAU_REF):
            p = [ct.leak_reversal, ct.tau * 1e3, ct.thresh, ct.reset]
        else:
            p = [ct.C, ct.leak_conductance * 1e-3, ct.leak_reversal, ct.thresh, ct.reset]
        if kind in (POINT_IAF_TAU_REF, POINT_IAF_REF):
            p.append(ct.refract * 1e3)
        return kind, p
    if isinstance(ct, AdExCell):
        return POINT_ADEX, [ct.C, ct.gL * 1e-3, ct.EL, ct.VT, ct.thresh, ct.reset, ct.delT, ct.tauw * 1e3,
                            ct.refract * 1e3, ct.a * 1e-3, ct.b]
    if isinstance(ct, IzhikevichCell):
        return POINT_IZH_DL, [ct.v0, ct.thresh, ct.a, ct.b, ct.c, ct.d]
    if isinstance(ct, FitzHughNagumoCell):
        return POINT_FN, [ct.I, 0.0]          # I, and V's value before the run (W starts at 0 too)
    raise ValueError(f"not a point neuron: {type(ct).__name__}")


def step_times_f32(dt: np.float32, n_steps: int) -> np.ndarray:
    """Float time (us) of steps 1..n_steps: the double sum of k - 1 float
    dts, as a float (eden/Eden.cpp:11486, 11931)."""
    acc = np.concatenate([[0.0], np.add.accumulate(np.full(max(n_steps - 1, 0), float(np.float32(dt))))])
    return acc[:n_steps].astype(F32)


def timed_steps(times_ms, th: np.ndarray) -> np.ndarray:
    """Steps (>= 1) in which a spike list fires, given th[n-1] = t_n + dt in
    float: the first step whose t + dt exceeds each time, once per step
    (eden/Eden.cpp:3759-3790)."""
    times = np.sort(ms_to_us(np.asarray(times_ms, np.float64)).astype(F32))
    idx = np.searchsorted(th, times, side="right")
    return (np.unique(idx[idx < len(th)]) + 1).astype(np.int64)


_MASK64 = (1 << 64) - 1
NOT_AN_INSTANCE = ~0xFEE1600D   # the `instance` of a cell's own LEMS code (eden/Eden.cpp:3255-3256)


def _hash64shift(key: int) -> int:
    key = ((~key) + (key << 21)) & _MASK64
    key ^= key >> 24
    key = (key + (key << 3) + (key << 8)) & _MASK64
    key ^= key >> 14
    key = (key + (key << 2) + (key << 4)) & _MASK64
    key ^= key >> 28
    return (key + (key << 31)) & _MASK64


def randof(x, work_item: int, instance: int, step: int, invocation: int) -> np.float32:
    """The reference's random(x) (eden/Eden.cpp:3216-3233): x times a 23-bit
    uniform from the integer hash of (work item, instance, step, call id)."""
    hi = ((int(work_item) << 24) | (int(instance) & 0xFFFFFF)) & _MASK64
    lo = ((int(invocation) << 40) | (int(step) & ((1 << 40) - 1))) & _MASK64
    sample = _hash64shift(_hash64shift(lo) ^ hi)
    r = F32(sample % (1 << 23)) / F32(1 << 23)
    return F32(F32(x) * F32(r))


def random_source_steps(ct, seed: int, tk: np.ndarray) -> np.ndarray:
    """Steps (1-based) in which a spikeGeneratorRandom / spikeGeneratorPoisson
    / spikeGeneratorRefPoisson emits (LEMS_CoreComponents.inc.xml:778-930 as
    the reference's LEMS code runs them, eden/Eden.cpp:2832-2994): the
    OnStart draw of the last initialisation pass (step 0, call id 0) sets
    the first spike time; a step whose float time exceeds it emits, draws
    the next interval (step n, call id 1) and moves the spike time on."""
    n_steps = len(tk)
    us = F32(1000.0)

    def first_after(n0, tnext):
        # first step >= n0 (1-based) whose time exceeds tnext
        return max(n0, int(np.searchsorted(tk, tnext, side="right")) + 1)

    fire = []
    with np.errstate(all="ignore"):
        if isinstance(ct, SpikeGeneratorRandomCell):
            lo, hi = _to_f32(ct.min_isi * 1000.0), _to_f32(ct.max_isi * 1000.0)
            x = F32(F32(hi - lo) / us)
            draw = lambda n, inv: F32(lo + F32(us * randof(x, seed, NOT_AN_INSTANCE, n, inv)))
            tnext = draw(0, 0)
            n = first_after(1, tnext)
            while n <= n_steps:
                fire.append(n)
                tnext = F32(tnext + draw(n, 1))
                n = first_after(n + 1, tnext)
        else:
            rate = _to_f32(ct.rate * 1e-6)
            if ct.min_isi is None:
                draw = lambda n, inv: F32(F32(F32(-1.0) * np.log(randof(1.0, seed, NOT_AN_INSTANCE, n, inv))) / rate)
            else:
                mi = _to_f32(ct.min_isi * 1000.0)
                avg = F32(F32(1.0) / rate)
                draw = lambda n, inv: F32(mi - F32(F32(avg - mi) *
                                                   np.log(randof(1.0, seed, NOT_AN_INSTANCE, n, inv))))
            small = F32(1e-6)   # SMALL_TIME, 1e-9 ms in us
            t_ideal = t_used = draw(0, 0)
            n = first_after(1, t_used)
            while n <= n_steps:
                fire.append(n)
                t = tk[n - 1]
                t_ideal = F32(t_ideal + draw(n, 1))
                h1 = F32(0.0) if F32(F32(t_ideal - t) / t) < 0 else F32(1.0)
                h2 = F32(0.0) if F32(F32(t - t_ideal) / t) < 0 else F32(1.0)
                t_used = F32(F32(t_ideal * h1) + F32(F32(t + small) * h2))
                if not np.isfinite(t_used):
                    break
                n = first_after(n + 1, t_used)
    return np.asarray(fire, np.int64)


def spike_source_steps(ext_cells: dict, dt: np.float32, n_steps: int, seeds: np.ndarray = None):
    """(source, logging step) of every spike the spike sources emit in steps
    1..n_steps, in step order and by source within a step.  A step n emits
    when it crosses the next spike time: spikeArray (the reference's spike
    list, eden/Eden.cpp:6738-6790) when the next listed time T < t_n + dt
    in float, consuming every such time; spikeGenerator
    (LEMS_CoreComponents.inc.xml:739-777) when tnext - t_n < 1e-9 ms, then
    tnext += period (tnext = period at the start).  The spike is logged at
    step n + 1, like a cell's threshold crossing."""
    tk = step_times_f32(dt, n_steps)
    th = (tk + F32(dt)).astype(F32)          # t_n + dt, in float
    srcs, steps = [], []
    for ct, gids in ext_cells.values():
        if isinstance(ct, EventSetReaderCell):
            s_, k_ = event_set_steps(ct, gids, dt, n_steps)
            srcs.append(s_)
            steps.append(k_)
            continue
        if isinstance(ct, (SpikeGeneratorRandomCell, SpikeGeneratorPoissonCell)):
            for g in gids:
                fire = random_source_steps(ct, int(seeds[g]), tk)
                srcs.append(np.full(len(fire), g, np.int32))
                steps.append(fire + 1)
            continue
        if isinstance(ct, SpikeArrayCell):
            times = np.sort(ms_to_us(np.asarray(ct.times, np.float64)).astype(F32))
            idx = np.searchsorted(th, times, side="right")   # first n - 1 with T < t_n + dt
            fire = np.unique(idx[idx < n_steps]) + 1
        else:
            period = F32(ct.period * 1000.0)
            small = F32(1e-6)
            fire = []
            tnext = period
            for n in range(1, n_steps + 1):
                if F32(tnext - tk[n - 1]) < small:
                    fire.append(n)
                    tnext = F32(tnext + period)
            fire = np.asarray(fire, np.int64)
        for g in gids:
            srcs.append(np.full(len(fire), g, np.int32))
            steps.append(fire.astype(np.int64) + 1)
    if not srcs:
        return np.zeros(0, np.int32), np.zeros(0, np.int64)
    src = np.concatenate(srcs)
    step = np.concatenate(steps)
    order = np.lexsort((src, step))
    return src[order], step[order]


def event_set_steps(ct, gids, dt: np.float32, n_steps: int):
    """(source, logging step) of an event-set reader's events
    (eden/Eden.cpp:11760-11829).  Frames whose timestamp does not exceed the
    last accepted one are ignored, as are negative timestamps; a frame is
    applied in the first step n whose double time satisfies
    timestamp < max(t_n - 1e-9 s, 0), raising its sources' trigger flags
    before the step's work items run, so their synapses read them in that
    same step -- in this library's terms a spike logged at step n."""
    gids = np.asarray(gids, np.int64)
    tn = np.concatenate([[0.0], np.add.accumulate(np.full(max(n_steps - 1, 0), float(np.float32(dt))))])[:n_steps]
    until = np.maximum(tn - 1e-3, 0.0)           # us
    src, step = [], []
    last = -np.inf
    n_ports = len(ct.ports)
    for ts_s, pairs in ct.frames:
        ts = ts_s * 1e6
        if not ts > last:
            continue
        last = ts
        if ts < 0 or not pairs:
            continue
        n = int(np.searchsorted(until, ts, side="right")) + 1   # first step with ts < until
        if n > n_steps:
            continue
        for inst, port in pairs:
            src.append(int(gids[int(inst) * n_ports + int(port)]))
            step.append(n)
    if not src:
        return np.zeros(0, np.int32), np.zeros(0, np.int64)
    pairs_ = np.unique(np.stack([np.asarray(step, np.int64), np.asarray(src, np.int64)], 1), axis=0)
    return pairs_[:, 1].astype(np.int32), pairs_[:, 0]


def poisson_rng_bases(spec: NetworkSpec, gid_ctype: np.ndarray, gid_is_point: np.ndarray) -> list:
    """Per Poisson component of `spec`, the random-call id of each of its
    inputs' first draw.  The reference numbers a cell type's random() calls
    as it generates code: compartment by compartment (eden/Eden.cpp:6540,
    the compartment's offset is the count so far), and within a compartment
    one code block per input component present on it in any cell of the
    type, in the order the components are defined (eden/Eden.cpp:1812-1830,
    5943), each Poisson block making two calls (eden/Eden.cpp:2450-2458)."""
    if not spec.poissons:
        return []
    span = 1 << 20
    keys = []
    for po in spec.poissons:
        cells = np.asarray(po.cell, np.int64)
        local = np.where(gid_is_point[cells], 0, np.asarray(po.seg, np.int64))
        keys.append(gid_ctype[cells].astype(np.int64) * span + local)
    # the Poisson components on each (cell type, compartment)
    present = {}
    for k, kk in enumerate(keys):
        for key in np.unique(kk).tolist():
            present.setdefault(key, []).append(k)
    offset = {}
    for key in sorted(present):
        ty = key // span
        prev = offset.get(("end", ty), 0)
        offset[key] = prev
        offset[("end", ty)] = prev + 2 * len(present[key])
    out = []
    for k, kk in enumerate(keys):
        uniq, inv = np.unique(kk, return_inverse=True)
        base = np.array([offset[key] + 2 * present[key].index(k) for key in uniq.tolist()], np.int64)
        out.append(base[inv].astype(np.int32) if len(kk) else np.zeros(0, np.int32))
    return out


def joined(parts, dtype) -> np.ndarray:
    return np.concatenate(parts).astype(dtype) if parts else np.zeros(0, dtype)


def _split_exp_three(spec):
    """A copy of `spec` in which each expThreeSynapse is two expTwo
    components in its place, `<name>:1` (gbase1, tauRise, tauDecay1) and
    `<name>:2` (gbase2, tauRise, tauDecay2), and each of its connections and
    timed inputs one of each.  Its conductance gbase1 (B - A) + gbase2 (C - A)
    with A jumping by (gbase1 wf1 + gbase2 wf2) / (gbase1 + gbase2)
    (LEMS_CoreComponents.inc.xml:182-224) is, A's decay being linear, the
    sum of the two expTwo conductances gbase_k (B_k - A_k) whose A_k jump by
    wf_k: the same waveform factors, the shared rise time and erev.  A
    Poisson input draws one spike train, so it cannot be split; it is
    refused on an expThreeSynapse."""
    import copy
    import dataclasses
    plastic = {s.name for s in spec.synapses if s.kind == SYN_BLOCKING_PLASTIC}
    for inp in list(spec.poissons) + list(spec.timed):
        if inp.synapse in plastic:
            raise ValueError(f"blockingPlasticSynapse {inp.synapse} on an input: connections only")
    three = {s.name: s for s in spec.synapses if s.kind == SYN_EXPTHREE}
    if not three:
        return spec
    for po in spec.poissons:
        if po.synapse in three:
            raise ValueError(f"Poisson input on expThreeSynapse {po.synapse}: not supported")
    out = copy.copy(spec)
    out.synapses = []
    for s in spec.synapses:
        if s.kind != SYN_EXPTHREE:
            out.synapses.append(s)
            continue
        for k, (g, td) in enumerate(((s.gbase, s.tau_decay), (s.gbase2, s.tau_decay2)), 1):
            out.synapses.append(SynapseType(f"{s.name}:{k}", SYN_EXPTWO, g, s.erev, td, s.tau_rise))
    out.projections = []
    for pr in spec.projections:
        if pr.synapse not in three:
            out.projections.append(pr)
            continue
        for k in (1, 2):
            out.projections.append(dataclasses.replace(pr, name=f"{pr.name}:{k}", synapse=f"{pr.synapse}:{k}"))
    out.timed = []
    for ti in spec.timed:
        if ti.synapse not in three:
            out.timed.append(ti)
            continue
        for k in (1, 2):
            out.timed.append(dataclasses.replace(ti, synapse=f"{ti.synapse}:{k}"))
    return out


EDEN_SYN_BLOCKING_PLASTIC = 5   # the library's kind number of a blockingPlasticSynapse

CABLE_BWD_EULER = 0
CABLE_FWD_EULER = 1


def _cable_solver(spec) -> int:
    """The model's cable solver: the reference's `cable_solver` setting,
    where `auto` means backward Euler (eden/Eden.cpp:4699-4702)."""
    name = getattr(spec, "cable_solver", "auto")
    if name not in ("auto", "bwd_euler", "fwd_euler"):
        raise ValueError(f"cable solver {name!r} unknown (auto, bwd_euler or fwd_euler)")
    return CABLE_FWD_EULER if name == "fwd_euler" else CABLE_BWD_EULER


def lower(spec: NetworkSpec) -> LoweredModel:
    if spec.custom_setup:
        from .custom_setup import apply_inputs, apply_synapses
        spec = apply_synapses(apply_inputs(spec))
    spec = _split_exp_three(spec)
    dt = _to_f32(spec.dt * 1000.0)
    gid_off = spec.pop_offsets()
    n_cells = spec.n_cells

    # ---- channel types ------------------------------------------------------
    chan_types = np.zeros(len(spec.channels), dtype=CHAN_DTYPE)
    for k, ch in enumerate(spec.channels):
        ct = chan_types[k]
        if len(ch.gates) > MAX_GATES:
            raise ValueError(f"channel {ch.name}: more than {MAX_GATES} gates")
        ct["n_gates"] = len(ch.gates)
        for g, gate in enumerate(ch.gates):
            ct["gate_instances"][g] = gate.instances
            if gate.kind not in GATE_KINDS:
                raise ValueError(f"channel {ch.name} gate {gate.name}: unknown kind {gate.kind!r}")
            needs = {"rates": (1, 0, 0), "tauInf": (0, 1, 1), "ratesTau": (1, 1, 0), "ratesInf": (1, 0, 1),
                     "ratesTauInf": (1, 1, 1), "instantaneous": (0, 0, 1)}[gate.kind]
            have = (gate.forward is not None and gate.reverse is not None, gate.tau is not None, gate.inf is not None)
            if tuple(bool(x) for x in needs) != have:
                want = [n for n, k in zip(("forward/reverse rates", "timeCourse", "steadyState"), needs) if k]
                raise ValueError(f"channel {ch.name} gate {gate.name}: a {gate.kind} gate has exactly "
                                 f"{', '.join(want)}")
            if gate.forward is not None:
                ct["fwd_kind"][g] = gate.forward.kind
                ct["fwd_rate"][g] = _to_f32(gate.forward.rate * 1e-3)   # per_ms -> per_us
                ct["fwd_mid"][g] = _to_f32(gate.forward.midpoint)
                ct["fwd_scale"][g] = _to_f32(gate.forward.scale)
                ct["rev_kind"][g] = gate.reverse.kind
                ct["rev_rate"][g] = _to_f32(gate.reverse.rate * 1e-3)
                ct["rev_mid"][g] = _to_f32(gate.reverse.midpoint)
                ct["rev_scale"][g] = _to_f32(gate.reverse.scale)
            ct["q10"][g] = gate_q10(gate, spec.temperature)
            ct["gate_kind"][g] = GATE_KINDS[gate.kind]
            if gate.tau is not None:      # fixedTimeCourse: tau in us
                ct["tau_kind"][g] = RATE_FIXED
                ct["tau_rate"][g] = _to_f32(gate.tau * 1000.0)
            if gate.inf is not None:      # HH*Variable: dimensionless
                ct["inf_kind"][g] = gate.inf.kind
                ct["inf_rate"][g] = _to_f32(gate.inf.rate)
                ct["inf_mid"][g] = _to_f32(gate.inf.midpoint)
                ct["inf_scale"][g] = _to_f32(gate.inf.scale)

    # ---- cells, in gid order ------------------------------------------------
    phys_off = [0]
    comp_parent, comp_c, comp_r, comp_area, comp_inv, comp_v0 = [], [], [], [], [], []
    chan_off = [np.zeros(1, np.int64)]     # per cell: arrays, joined at the end
    chan_type, chan_g, chan_e = [], [], []
    chan_dens, phys_ra = [], []
    chan_cache, chan_count = {}, [0]
    izh_kind = []
    ext_cells = {}                         # spike-source cell type -> (type, gids)
    izh = []
    src_target = np.zeros(n_cells, np.int32)
    src_thr = np.full(n_cells, np.nan, np.float32)
    gid_base = np.zeros(n_cells, np.int64)
    gid_is_izh = np.zeros(n_cells, bool)
    izh_index = np.full(n_cells, -1, np.int64)
    no_current = np.zeros(n_cells, bool)
    dl_cell = np.zeros(n_cells, bool)      # cells whose input current is dimensionless (izhikevichCell)
    geom_cache = {}
    gid_ctype = np.zeros(n_cells, np.int32)
    ctype_index = {c.name: k for k, c in enumerate(spec.cells)}
    from .custom_setup import apply_to, overrides
    setup = overrides(spec) if spec.custom_setup else {}
    gid = 0
    for pop in spec.populations:
        ct_pop = spec.cell_type(pop.cell_type)
        gid_ctype[gid:gid + pop.size] = ctype_index[ct_pop.name]
        for inst in range(pop.size):
            ct = apply_to(ct_pop, setup[(pop.name, inst)]) if (pop.name, inst) in setup else ct_pop
            if isinstance(ct, PhysicalCell):
                if ct.name not in geom_cache:
                    geom_cache[ct.name] = _cable_geometry(ct)
                c, r, a, inv = geom_cache[ct.name]
                base = phys_off[-1]
                gid_base[gid] = base
                comp_parent.append(np.asarray(ct.seg_parent, np.int32))
                comp_c.append(c)
                comp_r.append(r)
                comp_area.append(a)
                comp_inv.append(inv)
                comp_v0.append(np.full(ct.n_seg, _to_f32(ct.v0), np.float32))
                if ct.name not in chan_cache:
                    # channels segment by segment, densities in declaration order
                    if ct.densities:
                        mask = np.stack([np.asarray(d.seg_mask, bool) for d in ct.densities])  # [D, n_seg]
                        seg_i, kd = np.nonzero(mask.T)
                    else:
                        seg_i = kd = np.zeros(0, np.int64)
                    per_seg = np.bincount(seg_i, minlength=ct.n_seg)
                    dd = ct.densities
                    chan_cache[ct.name] = (kd.astype(np.int32),
                                           np.array([dd[k].channel for k in range(len(dd))], np.int32)[kd],
                                           np.array([dd[k].cond for k in range(len(dd))], np.float64)[kd],
                                           np.array([dd[k].erev for k in range(len(dd))], np.float64)[kd],
                                           np.cumsum(per_seg))
                kd_c, ty_c, g_c, e_c, ends = chan_cache[ct.name]
                n_before = chan_count[0]
                chan_dens.append(kd_c)
                chan_type.append(ty_c)
                chan_g.append(g_c)
                chan_e.append(e_c)
                chan_off.append(n_before + ends)
                chan_count[0] += len(kd_c)
                phys_off.append(base + ct.n_seg)
                phys_ra.append(float(ct.ra))
                src_target[gid] = base  # segment 0 detects spikes
                src_thr[gid] = _to_f32(ct.spike_thresh)
            elif isinstance(ct, SPIKE_SOURCE_TYPES):
                # a source with no target: its spikes are computed here
                src_target[gid] = -1
                gid_base[gid] = -1
                ext_cells.setdefault(ct.name, (ct, []))[1].append(gid)
            elif isinstance(ct, (Izhikevich2007Cell, IafCell, AdExCell, IzhikevichCell, FitzHughNagumoCell)):
                gid_is_izh[gid] = True
                izh_index[gid] = len(izh)
                kind, params = point_params(ct)
                no_current[gid] = kind in (POINT_IAF_TAU, POINT_IAF_TAU_REF, POINT_FN)
                dl_cell[gid] = kind == POINT_IZH_DL
                izh.append(params + [0.0] * (POINT_PARAMS - len(params)))
                izh_kind.append(kind)
            else:
                raise ValueError(f"unsupported cell type {type(ct).__name__}")
            gid += 1
    n_comp = phys_off[-1]
    for g in np.nonzero(gid_is_izh)[0]:
        gid_base[g] = n_comp + izh_index[g]
        src_target[g] = n_comp + izh_index[g]

    def target_of(gids, segs, current=True, dimensionless=False):
        gids = np.asarray(gids, np.int64)
        segs = np.asarray(segs, np.int64)
        if len(gids) and (gid_base[gids] < 0).any():
            raise ValueError("a spike source (spikeArray, spikeGenerator) has no membrane to target")
        if current and len(gids) and no_current[gids].any():
            raise ValueError("iafTauCell and iafTauRefCell do not receive current (synapses or inputs)")
        if current and len(gids) and (dl_cell[gids] != dimensionless).any():
            raise ValueError("izhikevichCell takes the dimensionless inputs (pulse/sine/rampGeneratorDL) only, "
                             "and those drive no other cell")
        t = gid_base[gids] + np.where(gid_is_izh[gids], 0, segs)
        return t.astype(np.int32)

    ext_src, ext_step = spike_source_steps(ext_cells, dt, spec.n_steps(), cell_seeds(spec.seed, n_cells))

    # ---- synapse types --------------------------------------------------------
    syn_types = np.zeros(len(spec.synapses), dtype=SYN_DTYPE)
    syn_index = {}
    for k, s in enumerate(spec.synapses):
        syn_index[s.name] = k
        st = syn_types[k]
        st["kind"] = EDEN_SYN_BLOCKING_PLASTIC if s.kind == SYN_BLOCKING_PLASTIC else s.kind
        # nS -> uS; the current-based kinds' jumps stay in nA
        st["gbase"] = (_to_f32(s.gbase) if s.kind in (SYN_ALPHA_CURRENT, SYN_EXPONE_CURRENT)
                       else _to_f32(s.gbase * 1e-3))
        st["erev"] = _to_f32(s.erev)
        st["tau_decay"] = _to_f32(s.tau_decay * 1000.0)
        two = s.kind in (SYN_EXPTWO, SYN_BLOCKING_PLASTIC)
        st["tau_rise"] = _to_f32(s.tau_rise * 1000.0) if two else 0.0
        st["waveform_factor"] = exptwo_waveform_factor(st["tau_rise"], st["tau_decay"]) if two else 1.0
        st["weight_prop"] = 1.0
        if s.kind == SYN_BLOCKING_PLASTIC:
            if s.plasticity:
                st["release_prob"] = _to_f32(s.plasticity["initReleaseProb"])
                st["tau_rec"] = _to_f32(s.plasticity["tauRec"] * 1000.0)
                st["tau_fac"] = _to_f32(s.plasticity.get("tauFac", 0.0) * 1000.0)
            if s.block:
                st["block_ratio"] = _to_f32(s.block["blockConcentration"] / s.block["scalingConc"])
                st["block_volt"] = _to_f32(s.block["scalingVolt"])

    # ---- gap junctions: each electrical connection puts an instance on both
    # ends, each taking weight * conductance * (V_peer - V_own) as synaptic
    # current (eden/Eden.cpp:9233-9251, 3407-3422); physical compartments only
    # A continuous connection puts its postComponent on the post end, then
    # its preComponent on the pre end (eden/Eden.cpp:9254-9270): a
    # linearGradedSynapse end is a gap-junction end, a gradedSynapse end
    # has its own state (graded_*), a silentSynapse end is nothing.
    gap_of = {g.name: g for g in spec.gap_types}
    gj_t, gj_p, gj_g, gj_w = [], [], [], []
    gr_t, gr_p, gr_par, gr_w = [], [], [], []

    def put_end(comp, at, peer, w):
        gt = gap_of[comp]
        if gt.kind == "silentSynapse":
            return
        if gt.kind == "gradedSynapse":
            gr_t.append(at); gr_p.append(peer); gr_w.append(w)
            gr_par.append([_to_f32(gt.conductance * 1e-3), _to_f32(gt.delta), _to_f32(gt.k * 1e-3),
                           _to_f32(gt.vth), _to_f32(gt.erev)])   # uS, mV, 1/us, mV, mV
            return
        gj_t.append(at); gj_p.append(peer); gj_w.append(w)
        gj_g.append(_to_f32(gt.conductance * 1e-3))   # nS -> uS

    def ends_of(name, pre_cell, pre_seg, post_cell, post_seg, weight):
        pre = np.asarray(pre_cell, np.int64)
        post = np.asarray(post_cell, np.int64)
        if len(pre) and (gid_is_izh[pre].any() or gid_is_izh[post].any()):
            raise ValueError(f"{name}: electrical and continuous connections join compartments of physical cells")
        return (target_of(pre, pre_seg, current=False), target_of(post, post_seg, current=False),
                np.asarray(weight, np.float64).astype(F32))

    for ep in spec.electrical:
        a, b, w = ends_of(ep.name, ep.pre_cell, ep.pre_seg, ep.post_cell, ep.post_seg, ep.weight)
        for i in range(len(a)):
            put_end(ep.synapse, a[i], b[i], w[i])
            put_end(ep.synapse, b[i], a[i], w[i])
    for cp in spec.continuous:
        a, b, w = ends_of(cp.name, cp.pre_cell, cp.pre_seg, cp.post_cell, cp.post_seg, cp.weight)
        for i in range(len(a)):
            put_end(cp.post_component, b[i], a[i], w[i])
            put_end(cp.pre_component, a[i], b[i], w[i])

    # ---- connection synapses: grouped per target, type order, then connection order
    tgt, typ, src, wgt, dly, order_key = [], [], [], [], [], []
    seq = 0
    for pr in spec.projections:
        k = syn_index[pr.synapse]
        n = len(pr.pre_cell)
        tgt.append(target_of(pr.post_cell, pr.post_seg))
        typ.append(np.full(n, k, np.int32))
        src.append(np.asarray(pr.pre_cell, np.int32))
        wgt.append(np.asarray(pr.weight, np.float64).astype(F32))
        dly.append(ms_to_us(pr.delay).astype(F32))
        order_key.append(np.arange(seq, seq + n, dtype=np.int64))
        seq += n
    if tgt:
        tgt = np.concatenate(tgt); typ = np.concatenate(typ); src = np.concatenate(src)
        wgt = np.concatenate(wgt); dly = np.concatenate(dly); order_key = np.concatenate(order_key)
        perm = np.lexsort((order_key, typ, tgt))
        tgt, typ, src, wgt, dly = tgt[perm], typ[perm], src[perm], wgt[perm], dly[perm]
    else:
        tgt = np.zeros(0, np.int32); typ = np.zeros(0, np.int32); src = np.zeros(0, np.int32)
        wgt = np.zeros(0, F32); dly = np.zeros(0, F32)

    # ---- poisson inputs -----------------------------------------------------
    pt, pty, pr_, pw, ps, pinst, prng = [], [], [], [], [], [], []
    rng_base = poisson_rng_bases(spec, gid_ctype, gid_is_izh)
    for k_po, po in enumerate(spec.poissons):
        k = syn_index[po.synapse]
        cells = np.asarray(po.cell, np.int64)
        segs = np.asarray(po.seg, np.int64)
        t = target_of(cells, segs)
        # instance number within each (cell, compartment) table, in input order
        inst = np.zeros(len(cells), np.int32)
        counter = {}
        for i in range(len(cells)):
            key = int(t[i])
            inst[i] = counter.get(key, 0)
            counter[key] = inst[i] + 1
        pt.append(t); pty.append(np.full(len(cells), k, np.int32))
        pr_.append(np.full(len(cells), _to_f32(po.rate * 1e-6), F32))
        pw.append(np.ones(len(cells), F32)); ps.append(cells.astype(np.int32)); pinst.append(inst)
        prng.append(rng_base[k_po])
    cat = lambda xs, dt_: (np.concatenate(xs) if xs else np.zeros(0, dt_))
    pt, pty, pr_, pw, ps, pinst = (cat(pt, np.int32), cat(pty, np.int32), cat(pr_, F32),
                                   cat(pw, F32), cat(ps, np.int32), cat(pinst, np.int32))
    prng = cat(prng, np.int32)
    if len(pt):
        perm = np.argsort(pt, kind="stable")
        pt, pty, pr_, pw, ps, pinst = pt[perm], pty[perm], pr_[perm], pw[perm], ps[perm], pinst[perm]
        prng = prng[perm]

    # ---- timed synaptic inputs: the steps each fires in -------------------------
    tm_t, tm_ty, tm_w, tm_off, tm_steps = [], [], [], [0], []
    if spec.timed:
        th = (step_times_f32(dt, spec.n_steps()) + F32(dt)).astype(F32)
        for ti in spec.timed:
            k = syn_index[ti.synapse]
            tm_t.append(target_of(ti.cell, ti.seg))
            tm_ty.append(np.full(len(ti.cell), k, np.int32))
            tm_w.append(np.asarray(ti.weight, np.float64).astype(F32))
            for times in ti.times:
                st = timed_steps(times, th)
                tm_steps.append(st)
                tm_off.append(tm_off[-1] + len(st))

    # ---- pulses ---------------------------------------------------------------
    qt, qs, qd, qa, qw = [], [], [], [], []
    for pu in spec.pulses:
        qt.append(target_of(pu.cell, pu.seg, dimensionless=pu.dimensionless))
        qs.append(ms_to_us(pu.delay).astype(F32))
        qd.append(ms_to_us(pu.duration).astype(F32))
        qa.append(np.asarray(pu.amplitude, np.float64).astype(F32))
        qw.append(np.ones(len(pu.cell), F32) if pu.weight is None else np.asarray(pu.weight, np.float64).astype(F32))
    qt, qs, qd, qa, qw = cat(qt, np.int32), cat(qs, F32), cat(qd, F32), cat(qa, F32), cat(qw, F32)
    if len(qt):
        perm = np.argsort(qt, kind="stable")
        qt, qs, qd, qa, qw = qt[perm], qs[perm], qd[perm], qa[perm], qw[perm]

    # ---- sine / ramp generators ----------------------------------------------
    wt, wsh, wpar, wwt = [], [], [], []
    for wv in spec.waves:
        if wv.shape not in WAVE_SHAPES:
            raise ValueError(f"unknown waveform input shape {wv.shape!r}")
        n = len(wv.cell)
        wt.append(target_of(wv.cell, wv.seg, dimensionless=wv.dimensionless))
        wsh.append(np.full(n, WAVE_SHAPES[wv.shape], np.int32))
        par = np.zeros((n, WAVE_PARAMS), np.float64)
        par[:, 0] = ms_to_us(wv.delay)
        par[:, 1] = ms_to_us(wv.duration)
        par[:, 2] = wv.p0
        par[:, 3] = ms_to_us(wv.p1) if wv.shape == WAVE_SINE else wv.p1
        par[:, 4] = wv.p2
        wpar.append(par.astype(F32))
        wwt.append(np.asarray(wv.weight, np.float64).astype(F32))
    wt, wsh, wwt = cat(wt, np.int32), cat(wsh, np.int32), cat(wwt, F32)
    wpar = np.concatenate(wpar) if wpar else np.zeros((0, WAVE_PARAMS), F32)
    if len(wt):
        perm = np.argsort(wt, kind="stable")
        wt, wsh, wpar, wwt = wt[perm], wsh[perm], wpar[perm], wwt[perm]

    # ---- voltage clamps ---------------------------------------------------------
    ct_, cpar, cwt = [], [], []
    for cl in spec.clamps:
        n = len(cl.cell)
        ct_.append(target_of(cl.cell, cl.seg))
        par = np.zeros((n, 6), np.float64)
        par[:, 0] = ms_to_us(cl.delay)
        par[:, 1] = ms_to_us(cl.duration)
        par[:, 2] = cl.v_before if cl.triple else np.nan
        par[:, 3] = cl.v_during
        par[:, 4] = cl.v_after if cl.triple else np.nan
        par[:, 5] = cl.resistance
        cpar.append(par.astype(F32))
        cwt.append(np.asarray(cl.weight, np.float64).astype(F32))
    ct_, cwt = cat(ct_, np.int32), cat(cwt, F32)
    cpar = np.concatenate(cpar) if cpar else np.zeros((0, 6), F32)
    if len(ct_):
        perm = np.argsort(ct_, kind="stable")
        ct_, cpar, cwt = ct_[perm], cpar[perm], cwt[perm]

    # a trace column records V of a target, or (code -2 - g) the state of gate
    # g, gates numbered channel instance by channel instance in comp_chan_off
    # order and within an instance in its type's gate order
    chan_off_all = np.concatenate(chan_off).astype(np.int64)
    chan_type_all = joined(chan_type, np.int32)
    chan_dens_all = joined(chan_dens, np.int32)
    gates_per_type = np.array([len(ch.gates) for ch in spec.channels] or [0], np.int64)
    gate_base = np.concatenate([[0], np.cumsum(gates_per_type[chan_type_all])]) if len(chan_type_all) else np.zeros(1)

    def trace_code(c):
        t = int(target_of([gid_off[c.pop] + c.cell], [c.seg], current=False)[0])
        if c.quantity == "v":
            return t
        dname, gname = c.quantity[2:].split("/")
        ct = spec.cell_type(spec.population(c.pop).cell_type)
        if not isinstance(ct, PhysicalCell):
            raise ValueError(f"recorded gate {c.quantity} of {c.pop}[{c.cell}]: not a physical cell")
        kd = [k for k, d in enumerate(ct.densities) if (d.name or f"cd{k}") == dname]
        if not kd:
            raise ValueError(f"recorded gate {c.quantity} of {c.pop}[{c.cell}]: no channelDensity {dname}")
        inst = [i for i in range(chan_off_all[t], chan_off_all[t + 1]) if chan_dens_all[i] == kd[0]]
        if not inst:
            raise ValueError(f"recorded gate {c.quantity}: channelDensity {dname} is not on segment {c.seg}")
        gnames = [g.name for g in spec.channels[chan_type_all[inst[0]]].gates]
        if gname not in gnames:
            raise ValueError(f"recorded gate {c.quantity}: the channel has no gate {gname}")
        return -2 - int(gate_base[inst[0]] + gnames.index(gname))
    trace_target = np.array([trace_code(c) for c in spec.trace_columns], dtype=np.int32)
    event_src = np.array([gid_off[e.pop] + e.cell for e in spec.event_selections], dtype=np.int32)

    izh_arr = np.asarray(izh, np.float64).astype(F32).reshape(-1, POINT_PARAMS)

    return LoweredModel(
        dt=dt, seed=int(spec.seed), n_steps=spec.n_steps(),
        phys_comp_off=np.asarray(phys_off, np.int32),
        comp_parent=cat(comp_parent, np.int32), comp_c=cat(comp_c, F32),
        comp_r_axial=cat(comp_r, F32), comp_area=cat(comp_area, F32),
        comp_inv_rc=cat(comp_inv, F32), comp_v0=cat(comp_v0, F32),
        chan_types=chan_types, comp_chan_off=np.concatenate(chan_off).astype(np.int32),
        chan_type=joined(chan_type, np.int32),
        chan_gbase=joined(chan_g, np.float64).astype(F32),
        chan_erev=joined(chan_e, np.float64).astype(F32),
        izh_params=izh_arr,
        src_target=src_target, src_threshold=src_thr,
        src_cell_seed=cell_seeds(spec.seed, n_cells),
        syn_types=syn_types, syn_target=tgt.astype(np.int32), syn_type=typ.astype(np.int32),
        syn_src=src.astype(np.int32), syn_weight=wgt.astype(F32), syn_delay=dly.astype(F32),
        pois_target=pt, pois_type=pty, pois_rate=pr_, pois_weight=pw, pois_src=ps,
        pois_instance=pinst,
        pulse_target=qt, pulse_start=qs, pulse_duration=qd, pulse_amplitude=qa,
        pulse_weight=qw,
        trace_target=trace_target, event_src=event_src, gid_target_base=gid_base,
        chan_density=joined(chan_dens, np.int32), phys_ra=np.asarray(phys_ra, np.float64),
        ext_src=ext_src, ext_step=ext_step, izh_kind=np.asarray(izh_kind, np.int32),
        timed_target=cat(tm_t, np.int32), timed_type=cat(tm_ty, np.int32), timed_weight=cat(tm_w, F32),
        timed_off=np.asarray(tm_off, np.int64), timed_step=cat(tm_steps, np.int64),
        wave_target=wt, wave_shape=wsh, wave_params=wpar, wave_weight=wwt,
        pois_rng_base=prng, clamp_target=ct_, clamp_params=cpar, clamp_weight=cwt,
        gap_target=np.asarray(gj_t, np.int32), gap_peer=np.asarray(gj_p, np.int32),
        gap_conductance=np.asarray(gj_g, F32), gap_weight=np.asarray(gj_w, F32),
        cable_solver=_cable_solver(spec),
        graded_target=np.asarray(gr_t, np.int32), graded_peer=np.asarray(gr_p, np.int32),
        graded_params=np.asarray(gr_par, F32).reshape(-1, 5), graded_weight=np.asarray(gr_w, F32),
    )


# ---------------------------------------------------------------------------
# ctypes mirror of include/eden_gpu.h
# ---------------------------------------------------------------------------
ABI_VERSION = 12
_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)


class CModel(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32), ("dt", ctypes.c_float), ("seed", ctypes.c_int64),
        ("n_phys", ctypes.c_int32), ("phys_comp_off", _i32p),
        ("n_comp", ctypes.c_int32), ("comp_parent", _i32p), ("comp_c", _f32p),
        ("comp_r_axial", _f32p), ("comp_area", _f32p), ("comp_inv_rc", _f32p), ("comp_v0", _f32p),
        ("n_chan_types", ctypes.c_int32), ("chan_types", ctypes.c_void_p),
        ("comp_chan_off", _i32p), ("chan_type", _i32p), ("chan_gbase", _f32p), ("chan_erev", _f32p),
        ("n_izh", ctypes.c_int32), ("izh_params", _f32p),
        ("n_src", ctypes.c_int32), ("src_target", _i32p), ("src_threshold", _f32p),
        ("src_cell_seed", _i32p),
        ("n_syn_types", ctypes.c_int32), ("syn_types", ctypes.c_void_p),
        ("n_syn", ctypes.c_int64), ("syn_target", _i32p), ("syn_type", _i32p),
        ("syn_src", _i32p), ("syn_weight", _f32p), ("syn_delay", _f32p),
        ("n_pois", ctypes.c_int64), ("pois_target", _i32p), ("pois_type", _i32p),
        ("pois_rate", _f32p), ("pois_weight", _f32p), ("pois_src", _i32p), ("pois_instance", _i32p),
        ("n_pulse", ctypes.c_int64), ("pulse_target", _i32p), ("pulse_start", _f32p),
        ("pulse_duration", _f32p), ("pulse_amplitude", _f32p), ("pulse_weight", _f32p),
        ("n_ext", ctypes.c_int64), ("ext_src", _i32p), ("ext_step", _i64p),
        ("izh_kind", _i32p),
        ("n_timed", ctypes.c_int64), ("timed_target", _i32p), ("timed_type", _i32p), ("timed_weight", _f32p),
        ("timed_off", _i64p), ("timed_step", _i64p),
        ("n_wave", ctypes.c_int64), ("wave_target", _i32p), ("wave_shape", _i32p), ("wave_params", _f32p),
        ("wave_weight", _f32p),
        ("pois_rng_base", _i32p),
        ("n_clamp", ctypes.c_int64), ("clamp_target", _i32p), ("clamp_params", _f32p), ("clamp_weight", _f32p),
        ("n_gap", ctypes.c_int64), ("gap_target", _i32p), ("gap_peer", _i32p), ("gap_conductance", _f32p),
        ("gap_weight", _f32p), ("cable_solver", ctypes.c_int32),
        ("n_graded", ctypes.c_int64), ("graded_target", _i32p), ("graded_peer", _i32p), ("graded_params", _f32p),
        ("graded_weight", _f32p),
    ]


def to_cmodel(m: LoweredModel):
    """Build the C struct; returns (struct, keepalive list of arrays)."""
    keep = []

    def p(arr, dtype, ptype):
        a = np.ascontiguousarray(arr, dtype=dtype)
        if a.size == 0:
            a = np.zeros(1, dtype=dtype)
        keep.append(a)
        return a.ctypes.data_as(ptype)

    def pv(arr):
        a = np.ascontiguousarray(arr)
        if a.size == 0:
            a = np.zeros(1, dtype=arr.dtype)
        keep.append(a)
        return ctypes.c_void_p(a.ctypes.data)

    cm = CModel()
    cm.abi_version = ABI_VERSION
    cm.dt = float(m.dt)
    cm.seed = int(m.seed)
    cm.n_phys = m.n_phys
    cm.phys_comp_off = p(m.phys_comp_off, np.int32, _i32p)
    cm.n_comp = m.n_comp
    cm.comp_parent = p(m.comp_parent, np.int32, _i32p)
    cm.comp_c = p(m.comp_c, F32, _f32p)
    cm.comp_r_axial = p(m.comp_r_axial, F32, _f32p)
    cm.comp_area = p(m.comp_area, F32, _f32p)
    cm.comp_inv_rc = p(m.comp_inv_rc, F32, _f32p)
    cm.comp_v0 = p(m.comp_v0, F32, _f32p)
    cm.n_chan_types = len(m.chan_types)
    cm.chan_types = pv(m.chan_types)
    cm.comp_chan_off = p(m.comp_chan_off, np.int32, _i32p)
    cm.chan_type = p(m.chan_type, np.int32, _i32p)
    cm.chan_gbase = p(m.chan_gbase, F32, _f32p)
    cm.chan_erev = p(m.chan_erev, F32, _f32p)
    cm.n_izh = m.n_izh
    cm.izh_params = p(m.izh_params.reshape(-1), F32, _f32p)
    cm.n_src = len(m.src_target)
    cm.src_target = p(m.src_target, np.int32, _i32p)
    cm.src_threshold = p(m.src_threshold, F32, _f32p)
    cm.src_cell_seed = p(m.src_cell_seed, np.int32, _i32p)
    cm.n_syn_types = len(m.syn_types)
    cm.syn_types = pv(m.syn_types)
    cm.n_syn = len(m.syn_target)
    cm.syn_target = p(m.syn_target, np.int32, _i32p)
    cm.syn_type = p(m.syn_type, np.int32, _i32p)
    cm.syn_src = p(m.syn_src, np.int32, _i32p)
    cm.syn_weight = p(m.syn_weight, F32, _f32p)
    cm.syn_delay = p(m.syn_delay, F32, _f32p)
    cm.n_pois = len(m.pois_target)
    cm.pois_target = p(m.pois_target, np.int32, _i32p)
    cm.pois_type = p(m.pois_type, np.int32, _i32p)
    cm.pois_rate = p(m.pois_rate, F32, _f32p)
    cm.pois_weight = p(m.pois_weight, F32, _f32p)
    cm.pois_src = p(m.pois_src, np.int32, _i32p)
    cm.pois_instance = p(m.pois_instance, np.int32, _i32p)
    cm.n_pulse = len(m.pulse_target)
    cm.pulse_target = p(m.pulse_target, np.int32, _i32p)
    cm.pulse_start = p(m.pulse_start, F32, _f32p)
    cm.pulse_duration = p(m.pulse_duration, F32, _f32p)
    cm.pulse_amplitude = p(m.pulse_amplitude, F32, _f32p)
    cm.pulse_weight = p(m.pulse_weight, F32, _f32p)
    cm.n_ext = len(m.ext_src)
    cm.ext_src = p(m.ext_src, np.int32, _i32p)
    cm.ext_step = p(m.ext_step, np.int64, _i64p)
    cm.izh_kind = p(m.izh_kind if m.izh_kind is not None and len(m.izh_kind) == m.n_izh
                    else np.zeros(m.n_izh, np.int32), np.int32, _i32p)
    cm.n_timed = len(m.timed_target)
    cm.timed_target = p(m.timed_target, np.int32, _i32p)
    cm.timed_type = p(m.timed_type, np.int32, _i32p)
    cm.timed_weight = p(m.timed_weight, F32, _f32p)
    cm.timed_off = p(m.timed_off, np.int64, _i64p)
    cm.timed_step = p(m.timed_step, np.int64, _i64p)
    cm.n_wave = len(m.wave_target)
    cm.wave_target = p(m.wave_target, np.int32, _i32p)
    cm.wave_shape = p(m.wave_shape, np.int32, _i32p)
    cm.wave_params = p(np.asarray(m.wave_params).reshape(-1), F32, _f32p)
    cm.wave_weight = p(m.wave_weight, F32, _f32p)
    if m.pois_rng_base is not None:
        cm.pois_rng_base = p(m.pois_rng_base, np.int32, _i32p)
    cm.n_clamp = len(m.clamp_target)
    cm.clamp_target = p(m.clamp_target, np.int32, _i32p)
    cm.clamp_params = p(np.asarray(m.clamp_params).reshape(-1), F32, _f32p)
    cm.clamp_weight = p(m.clamp_weight, F32, _f32p)
    cm.n_gap = len(m.gap_target)
    cm.gap_target = p(m.gap_target, np.int32, _i32p)
    cm.gap_peer = p(m.gap_peer, np.int32, _i32p)
    cm.gap_conductance = p(m.gap_conductance, F32, _f32p)
    cm.gap_weight = p(m.gap_weight, F32, _f32p)
    cm.cable_solver = int(m.cable_solver)
    cm.n_graded = len(m.graded_target)
    cm.graded_target = p(m.graded_target, np.int32, _i32p)
    cm.graded_peer = p(m.graded_peer, np.int32, _i32p)
    cm.graded_params = p(m.graded_params, F32, _f32p)
    cm.graded_weight = p(m.graded_weight, F32, _f32p)
    return cm, keep
