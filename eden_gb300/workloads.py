"""Seeded synthetic networks: the workloads this path is measured and tested on.

No public dataset exists for these runs; each generator draws a NeuroML
network of a stated shape from numpy's `default_rng(seed)`:

  single_comp_hh   1,000 single-compartment HH cells, one DC pulse each
                   (uniform 0-0.3 nA), no synapses, dt 0.025 ms, 1,000 ms.
  multicomp_net    10,000 cells with random branching trees (segment count
                   log-uniform in [1, 500], segment length 5-50 um, diameter
                   0.5-4 um, Ra 150 ohm*cm), HH soma + passive dendrites,
                   expTwoSynapse (0.5 / 5 ms, 1 nS, 0 mV) at fixed in-degree
                   100 with delays 0.5-5 ms, plus one 5 Hz poissonFiringSynapse
                   per synapse slot; dt 0.025 ms, 1,000 ms.
  izh_net          100,000 izhikevich2007Cell (80 % RS, 20 % FS), expOneSynapse
                   at in-degree 100 (lognormal weights, delays 1-20 ms in whole
                   steps), one DC pulse per cell; dt 0.1 ms, 1,000 ms.
  ball_and_stick   256 soma + 50-compartment HH cables with lognormal
                   per-instance parameters, 0.5 nA step for 150 ms;
                   dt 0.025 ms, 200 ms.
  mixed_scale      the multicomp and izhikevich populations together.
  spike_sources    spikeArray and spikeGenerator populations driving
                   izhikevich and single-compartment HH cells.
  event_sets       an EdenEventSetReader (spike events from a file, several
                   instances and ports) driving izhikevich and HH cells.
  point_neurons    iafTau, iafTauRef, iaf, iafRef and adExIaF cells with DC
                   pulses and recurrent expTwo / expOne synapses.
  timed_inputs     timedSynapticInput spike lists (expTwo and expOne) into
                   HH and izhikevich cells.
  input_kinds      every input kind on one branching cell type (HH soma,
                   passive dendrites) and on izhikevich cells: pulse, sine and
                   ramp generators, several Poisson components sharing
                   compartments, and timed inputs on passive dendrites.
  dl_inputs        izhikevichCell (dimensionless) driven by pulse, sine and
                   ramp generators of the DL kind, beside izhikevich2007
                   cells with the dimensional ones.
  custom_setup     izhikevich, iafRef and adExIaF populations whose
                   parameters an EdenCustomSetup file overrides per instance.
  random_sources   spikeGeneratorRandom, spikeGeneratorPoisson and
                   spikeGeneratorRefPoisson populations driving izhikevich
                   and HH cells.
  voltage_clamps   voltageClamp and voltageClampTriple on HH somata,
                   passive dendrites and izhikevich cells, with pulses.
  gap_junctions    gapJunction types of two conductances on soma-soma and
                   soma-dendrite electrical connections (weighted) between
                   single-compartment HH cells and branching cells, with DC
                   pulses on some somata and expTwo synapses onto coupled
                   compartments.
  alpha_synapses   alphaSynapse and alphaCurrentSynapse connections, Poisson
                   and timed inputs on HH somata and dendrites and
                   izhikevich2007 cells, beside expTwo connections.
  gate_kinds       channels with every built-in gate kind (gateHHrates,
                   gateHHtauInf, gateHHratesTau, gateHHratesInf,
                   gateHHratesTauInf), q10Fixed and q10ExpTemp settings at
                   16.3 degC, on single-compartment and branching cells.

Every generator takes scale arguments (cell count, in-degree, length) so the
same distributions produce the small cases the CPU reference can finish.
Delays are rounded to whole microseconds so that delivery times are exact
in single precision.
"""
from __future__ import annotations

import numpy as np

from .network import (RATE_EXP, RATE_EXPLINEAR, RATE_SIGMOID, AdExCell, Channel, ChannelDensity, EventSelection,
                      ClampInputs, FitzHughNagumoCell, Gate, IafCell, Izhikevich2007Cell, IzhikevichCell, Rate,
                      NetworkSpec, OutputColumn, PhysicalCell, PoissonInputs,
                      Population, Projection, PulseInputs, SpikeArrayCell, EventSetReaderCell,
                      SpikeGeneratorPoissonCell, SpikeGeneratorRandomCell,
                      SpikeGeneratorCell, SynapseType, SYN_EXPONE, SYN_EXPTWO, TimedInputs, WAVE_RAMP,
                      WAVE_SINE, WaveInputs, hh_channels, ElectricalProjection, GapJunctionType)

# conductivities (mS/cm2) and reversal potentials (mV) of the HH cells
G_NA, G_K, G_L = 120.0, 36.0, 0.3
E_NA, E_K, E_L = 50.0, -77.0, -54.387


def _hh_densities(n_seg: int, hh_mask: np.ndarray) -> list:
    allseg = np.ones(n_seg, dtype=bool)
    return [
        ChannelDensity(0, G_L, E_L, allseg),
        ChannelDensity(1, G_NA, E_NA, hh_mask.copy()),
        ChannelDensity(2, G_K, E_K, hh_mask.copy()),
    ]


def _round_us(delay_ms: np.ndarray) -> np.ndarray:
    return np.round(np.asarray(delay_ms) * 1000.0) / 1000.0


# ---------------------------------------------------------------------------
def single_comp_hh(n_cells: int = 1000, length_ms: float = 1000.0,
                   dt_ms: float = 0.025, seed: int = 1234,
                   n_recorded: int = 10) -> NetworkSpec:
    rng = np.random.default_rng(seed)
    cell = PhysicalCell(
        name="hhcell",
        seg_parent=np.array([-1]), seg_len=np.array([0.0]), seg_diam=np.array([17.8]),
        densities=_hh_densities(1, np.ones(1, dtype=bool)),
        cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0,
    )
    spec = NetworkSpec("single_comp_hh", dt_ms, length_ms, seed, channels=hh_channels())
    spec.cells.append(cell)
    spec.populations.append(Population("hhpop", "hhcell", n_cells))
    amp = np.round(rng.uniform(0.0, 0.3, n_cells), 6)
    spec.pulses.append(PulseInputs("*", np.arange(n_cells), np.zeros(n_cells, int),
                                   np.zeros(n_cells), np.full(n_cells, length_ms), amp))
    rec = np.sort(rng.choice(n_cells, size=min(n_recorded, n_cells), replace=False))
    spec.trace_columns = [OutputColumn("hhpop", int(c), 0) for c in rec]
    spec.event_selections = [EventSelection("hhpop", c, 0) for c in range(n_cells)]
    return spec


# ---------------------------------------------------------------------------
def random_tree(rng, n_seg: int, soma_len=20.0, soma_diam=20.0):
    """Random recursive tree: each new segment attaches to a uniformly chosen
    earlier one.  Segment 0 is a fixed-size cylindrical soma."""
    parent = np.empty(n_seg, dtype=np.int64)
    parent[0] = -1
    if n_seg > 1:
        parent[1:] = np.floor(rng.uniform(0, 1, n_seg - 1) * np.arange(1, n_seg)).astype(np.int64)
    length = np.round(rng.uniform(5.0, 50.0, n_seg), 3)
    diam = np.round(rng.uniform(0.5, 4.0, n_seg), 3)
    length[0], diam[0] = soma_len, soma_diam
    return parent, length, diam


def multicomp_net(n_cells: int = 10000, in_degree: int = 100, length_ms: float = 1000.0,
                  dt_ms: float = 0.025, seed: int = 1234, max_seg: int = 500,
                  poisson_rate_hz: float = 5.0, n_recorded: int = 10,
                  weight: float = 1.0, soma_diam: float = 20.0, hh_dend_frac: float = 0.0,
                  syn_on_dendrites: bool = False) -> NetworkSpec:
    """hh_dend_frac > 0 puts HH channels on that fraction of dendritic
    segments as well; syn_on_dendrites places each connection on a random
    segment of the target cell instead of the soma (both drawn from a second
    generator, so the default network is unchanged)."""
    rng = np.random.default_rng(seed)
    rng2 = np.random.default_rng(seed + 1)
    spec = NetworkSpec("multicomp_net", dt_ms, length_ms, seed, channels=hh_channels())
    syn = SynapseType("syn_e2", SYN_EXPTWO, gbase=1.0, erev=0.0, tau_decay=5.0, tau_rise=0.5)
    spec.synapses.append(syn)
    nseg = np.round(np.exp(rng.uniform(0.0, np.log(max_seg), n_cells))).astype(int)
    nseg = np.clip(nseg, 1, max_seg)
    for c in range(n_cells):
        parent, length, diam = random_tree(rng, int(nseg[c]), soma_diam=soma_diam, soma_len=soma_diam)
        soma = np.zeros(len(parent), dtype=bool)
        soma[0] = True
        hh = soma | (rng2.random(len(parent)) < hh_dend_frac) if hh_dend_frac > 0 else soma
        cell = PhysicalCell(f"mc{c}", parent, length, diam, _hh_densities(len(parent), hh),
                            cm=1.0, ra=150.0, v0=-65.0, spike_thresh=-20.0,
                            seg_groups={"soma_group": soma, "dend_group": ~soma})
        spec.cells.append(cell)
        spec.populations.append(Population(f"pop{c}", f"mc{c}", 1))
    # recurrent expTwo connections, fixed in-degree, presyn uniform over cells
    pre = rng.integers(0, n_cells, size=(n_cells, in_degree))
    delay = _round_us(rng.uniform(0.5, 5.0, size=(n_cells, in_degree)))
    post = np.repeat(np.arange(n_cells), in_degree)
    post_seg = None
    if syn_on_dendrites:
        nsegs = np.array([len(spec.cells[c].seg_parent) for c in range(n_cells)])
        post_seg = (rng2.random(post.size) * nsegs[post]).astype(int)
    spec.projections.append(_flat_projection(spec, "proj_e2", pre.ravel(), post, "syn_e2",
                                             np.full(post.size, weight), delay.ravel(), post_seg=post_seg))
    # one Poisson source per synapse slot, onto the soma
    if poisson_rate_hz > 0:
        spec.poissons.append(PoissonInputs("*", "syn_e2", poisson_rate_hz,
                                           np.repeat(np.arange(n_cells), in_degree),
                                           np.zeros(n_cells * in_degree, dtype=int)))
    rec = np.sort(rng.choice(n_cells, size=min(n_recorded, n_cells), replace=False))
    spec.trace_columns = [OutputColumn(f"pop{c}", 0, 0) for c in rec]
    spec.event_selections = [EventSelection(f"pop{c}", 0, 0) for c in range(n_cells)]
    return spec


def _flat_projection(spec, name, pre_gid, post_gid, synapse, weight, delay, post_seg=None):
    """A projection expressed on global cell ids; neuroml_io splits it per
    (pre, post) population pair when writing XML."""
    if post_seg is None:
        post_seg = np.zeros(len(post_gid), dtype=np.int64)
    return Projection(name, "*", "*", synapse, np.asarray(pre_gid, np.int64),
                      np.asarray(post_gid, np.int64), np.asarray(post_seg, np.int64),
                      np.asarray(weight, np.float64), np.asarray(delay, np.float64))


# ---------------------------------------------------------------------------
def izh_net(n_cells: int = 100000, in_degree: int = 100, length_ms: float = 1000.0,
            dt_ms: float = 0.1, seed: int = 1234, n_recorded: int = 10,
            pulse_max_na: float = 0.5) -> NetworkSpec:
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("izh_net", dt_ms, length_ms, seed)
    n_exc = int(round(0.8 * n_cells))
    n_inh = n_cells - n_exc
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.cells.append(Izhikevich2007Cell("izFS", a=0.1, d=0.0, c=-55.0))
    spec.populations.append(Population("exc", "izRS", n_exc))
    if n_inh:
        spec.populations.append(Population("inh", "izFS", n_inh))
    spec.synapses.append(SynapseType("syn_exc", SYN_EXPONE, gbase=1.0, erev=0.0, tau_decay=2.0))
    spec.synapses.append(SynapseType("syn_inh", SYN_EXPONE, gbase=1.0, erev=-80.0, tau_decay=5.0))
    pre = rng.integers(0, n_cells, size=(n_cells, in_degree)).ravel()
    post = np.repeat(np.arange(n_cells), in_degree)
    w = np.round(rng.lognormal(-1.0, 0.5, size=pre.size), 6)
    steps = rng.integers(10, 201, size=pre.size)
    delay = np.round(steps * dt_ms, 6)
    exc = pre < n_exc
    spec.projections.append(_flat_projection(spec, "proj_exc", pre[exc], post[exc], "syn_exc", w[exc], delay[exc]))
    spec.projections.append(_flat_projection(spec, "proj_inh", pre[~exc], post[~exc], "syn_inh", w[~exc], delay[~exc]))
    amp = np.round(rng.uniform(0.0, pulse_max_na, n_cells), 6)
    gids = np.arange(n_cells)
    spec.pulses.append(PulseInputs("*", gids, np.zeros(n_cells, int), np.zeros(n_cells),
                                   np.full(n_cells, length_ms), amp))
    rec = np.sort(rng.choice(n_cells, size=min(n_recorded, n_cells), replace=False))
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, int(g)), 0) for g in rec]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n_cells)]
    return spec


def routing_probe(n_arrays: int = 8, n_post: int = 16, fan_in: int = 40, length_ms: float = 30.0,
                  dt_ms: float = 0.1, seed: int = 1234, min_delay_ms: float = 0.1) -> NetworkSpec:
    """Spike lists into izhikevich2007 cells through expOne synapses, the
    case the per-synapse pending slots are compared on against the
    reference's own tables: spike trains with bursts closer together than
    the delays (a trigger read while a spike is pending is dropped or kept
    by the single-pending-spike rule), spikes on and next to step
    boundaries, and delays of whole and fractional steps (from
    `min_delay_ms`; below one step a spike fires in the step that reads
    its trigger).  The driven cells have no outgoing connections, so the
    spike trains reaching the synapses are the lists themselves."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("routing_probe", dt_ms, length_ms, seed)
    for k in range(n_arrays):
        base = rng.uniform(0.0, length_ms * 0.9, size=int(rng.integers(3, 8)))
        t = [base]
        for b in base[: len(base) // 2]:  # bursts: 2-3 more spikes 0.05-1 ms apart
            t.append(b + np.cumsum(rng.uniform(0.05, 1.0, size=int(rng.integers(2, 4)))))
        t = np.round(np.concatenate(t), 4)
        if k == 0:
            t = np.concatenate([t, [1.0, 1.0999, 1.1, 1.1001, 5.0, 5.05]])
        spec.cells.append(SpikeArrayCell(f"sa{k}", np.sort(t[t < length_ms])))
        spec.populations.append(Population(f"psa{k}", f"sa{k}", 1))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("iz", "izRS", n_post))
    spec.synapses.append(SynapseType("syn_e1", SYN_EXPONE, gbase=0.5, erev=0.0, tau_decay=2.0))
    post = np.repeat(np.arange(n_arrays, n_arrays + n_post), fan_in)
    pre = rng.integers(0, n_arrays, size=post.size)
    choices = np.array([1.0, 1.5, 2.0, 2.5, 3.0, 4.0, 7.0, 10.0, 13.3]) * min_delay_ms
    delay = _round_us(rng.choice(choices, size=post.size) + np.where(rng.random(post.size) < 0.3,
                                                                     rng.uniform(0.0, dt_ms, post.size), 0.0))
    w = np.round(rng.uniform(0.2, 1.0, size=post.size), 4)
    spec.projections.append(_flat_projection(spec, "proj", pre, post, "syn_e1", w, delay))
    spec.trace_columns = [OutputColumn("iz", 0, 0)]
    spec.event_selections = [EventSelection(f"psa{k}", 0, 0) for k in range(n_arrays)]
    return spec


def _gid_to_pop(spec, gid):
    """(population, index) of a global cell id."""
    n_pops = len(spec.populations)
    cache = spec.__dict__.setdefault("_gid_starts", {})
    starts = cache.get(n_pops)
    if starts is None:
        starts = np.concatenate([[0], np.cumsum([p.size for p in spec.populations])])
        cache.clear()
        cache[n_pops] = starts
    k = int(np.searchsorted(starts, gid, side="right")) - 1
    if gid < 0 or k >= n_pops:
        raise IndexError(gid)
    return spec.populations[k].name, int(gid - starts[k])


# ---------------------------------------------------------------------------
def ball_and_stick(n_inst: int = 256, n_dend: int = 50, length_ms: float = 200.0,
                   dt_ms: float = 0.025, seed: int = 1234, sigma: float = 0.3,
                   amp_na: float = 0.5, pulse_ms: float = 150.0,
                   params: np.ndarray | None = None, syn_drive: int = 0) -> NetworkSpec:
    """Per-instance parameters (7): soma gNa, gK, gL, dendrite gNa, gK, gL
    (mS/cm2) and Ra (ohm*cm), lognormal around the HH defaults.

    syn_drive > 0 adds synaptic drive whose events are fixed in advance, the
    case for synaptic-weight gradients: four spikeArray sources (seeded
    spike trains over the run) with syn_drive excitatory expTwoSynapse
    connections per cell (0.5 / 5 ms, 2 nS, 0 mV; weights 0.5-1.5, delays
    1-3 ms) onto random dendrite segments, and two inhibitory
    timedSynapticInput expOneSynapse inputs per cell (5 ms, 3 nS, -80 mV;
    weights 0.5-1.5) onto the soma.  They come from a second generator, so
    the cells and their parameters are those of the network without drive."""
    rng = np.random.default_rng(seed)
    base = np.array([G_NA, G_K, G_L, G_NA, G_K, G_L, 150.0])
    if params is None:
        params = np.round(base * rng.lognormal(0.0, sigma, size=(n_inst, 7)), 6)
    spec = NetworkSpec("ball_and_stick", dt_ms, length_ms, seed, channels=hh_channels())
    n_seg = 1 + n_dend
    parent = np.arange(-1, n_seg - 1, dtype=np.int64)
    seg_len = np.full(n_seg, 500.0 / n_dend)
    seg_diam = np.full(n_seg, 2.0)
    seg_len[0], seg_diam[0] = 20.0, 20.0
    soma = np.zeros(n_seg, dtype=bool)
    soma[0] = True
    for i in range(n_inst):
        p = params[i]
        dens = [
            ChannelDensity(0, p[2], E_L, soma.copy()), ChannelDensity(1, p[0], E_NA, soma.copy()),
            ChannelDensity(2, p[1], E_K, soma.copy()),
            ChannelDensity(0, p[5], E_L, ~soma), ChannelDensity(1, p[3], E_NA, ~soma),
            ChannelDensity(2, p[4], E_K, ~soma),
        ]
        spec.cells.append(PhysicalCell(f"bs{i}", parent.copy(), seg_len.copy(), seg_diam.copy(), dens,
                                       cm=1.0, ra=float(p[6]), v0=-65.0, spike_thresh=-20.0,
                                       seg_groups={"soma_group": soma, "dend_group": ~soma}))
        spec.populations.append(Population(f"pop{i}", f"bs{i}", 1))
    spec.pulses.append(PulseInputs("*", np.arange(n_inst), np.zeros(n_inst, int), np.zeros(n_inst),
                                   np.full(n_inst, pulse_ms), np.full(n_inst, amp_na)))
    if syn_drive:
        r2 = np.random.default_rng(seed + 7)
        spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=2.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
        spec.synapses.append(SynapseType("syn_i1", SYN_EXPONE, gbase=3.0, erev=-80.0, tau_decay=5.0))
        n_arr = 4
        for k in range(n_arr):
            t = np.round(np.sort(r2.uniform(0.0, length_ms, size=max(3, int(length_ms / 5)))), 4)
            spec.cells.append(SpikeArrayCell(f"sa{k}", t))
            spec.populations.append(Population(f"psa{k}", f"sa{k}", 1))
        post = np.repeat(np.arange(n_inst), syn_drive)
        pre = n_inst + r2.integers(0, n_arr, size=post.size)
        seg = r2.integers(1, n_seg, size=post.size)
        spec.projections.append(_flat_projection(spec, "proj_drive", pre, post, "syn_e2",
                                                 np.round(r2.uniform(0.5, 1.5, post.size), 4),
                                                 _round_us(r2.uniform(1.0, 3.0, post.size)), post_seg=seg))
        cells = np.repeat(np.arange(n_inst), 2)
        times = [np.round(np.sort(r2.uniform(0.0, length_ms, size=max(2, int(length_ms / 10)))), 4)
                 for _ in range(len(cells))]
        spec.timed.append(TimedInputs("syn_i1", cells, np.zeros(len(cells), np.int64), times,
                                      np.round(r2.uniform(0.5, 1.5, len(cells)), 4)))
    spec.trace_columns = [OutputColumn(f"pop{i}", 0, 0) for i in range(min(n_inst, 10))]
    spec.event_selections = [EventSelection(f"pop{i}", 0, 0) for i in range(n_inst)]
    spec.params = params
    return spec


# ---------------------------------------------------------------------------
def mixed_scale(n_izh: int = 160000, n_mc: int = 40000, in_degree: int = 100,
                length_ms: float = 1000.0, dt_ms: float = 0.025, seed: int = 1234,
                poisson_rate_hz: float = 2.0, n_seg: int = 100) -> NetworkSpec:
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("mixed_scale", dt_ms, length_ms, seed, channels=hh_channels())
    syn = SynapseType("syn_e2", SYN_EXPTWO, gbase=1.0, erev=0.0, tau_decay=5.0, tau_rise=0.5)
    spec.synapses.append(syn)
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("izh", "izRS", n_izh))
    for c in range(n_mc):
        parent, length, diam = random_tree(rng, n_seg)
        soma = np.zeros(n_seg, dtype=bool)
        soma[0] = True
        spec.cells.append(PhysicalCell(f"mc{c}", parent, length, diam, _hh_densities(n_seg, soma),
                                       cm=1.0, ra=150.0, seg_groups={"soma_group": soma, "dend_group": ~soma}))
        spec.populations.append(Population(f"pop{c}", f"mc{c}", 1))
    n = n_izh + n_mc
    pre = rng.integers(0, n, size=(n, in_degree)).ravel()
    post = np.repeat(np.arange(n), in_degree)
    delay = _round_us(rng.uniform(0.5, 10.0, size=pre.size))
    spec.projections.append(_flat_projection(spec, "proj_e2", pre, post, "syn_e2", np.full(pre.size, 0.2), delay))
    spec.poissons.append(PoissonInputs("*", "syn_e2", poisson_rate_hz, post.copy(), np.zeros(post.size, dtype=int)))
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


# ---------------------------------------------------------------------------
def spike_sources(n_arrays: int = 6, n_generators: int = 3, n_izh: int = 12, n_hh: int = 8,
                  fan_in: int = 6, length_ms: float = 100.0, dt_ms: float = 0.025, seed: int = 1234,
                  n_recorded: int = 6) -> NetworkSpec:
    """Spike sources with no membrane -- spikeArray populations (seeded
    spike times, some on and next to step boundaries, one list unsorted) and
    spikeGenerator populations (periods on and off the step grid) -- driving
    izhikevich2007 and single-compartment HH cells through expTwo and expOne
    synapses; the driven cells also connect among themselves."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("spike_sources", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=2.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    spec.synapses.append(SynapseType("syn_e1", SYN_EXPONE, gbase=3.0, erev=0.0, tau_decay=2.0))
    for k in range(n_arrays):
        t = np.round(np.sort(rng.uniform(0.0, length_ms, size=rng.integers(5, 40))), 4)
        if k == 0:   # step boundaries: on the grid, a hair before and after, and a duplicate
            t = np.concatenate([t, [0.0, 10.0, 10.0, 9.9999, 10.0001, 20.025]])
        if k == 1:   # listed out of order
            t = t[::-1].copy()
        spec.cells.append(SpikeArrayCell(f"sa{k}", t))
        spec.populations.append(Population(f"psa{k}", f"sa{k}", int(rng.integers(1, 4))))
    for k, period in enumerate([2.3, 3.7, 5.0, 1.025, 7.77][:n_generators]):
        spec.cells.append(SpikeGeneratorCell(f"sg{k}", period))
        spec.populations.append(Population(f"psg{k}", f"sg{k}", 2))
    n_src = sum(p.size for p in spec.populations)
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("iz", "izRS", n_izh))
    hh = PhysicalCell(name="hhcell", seg_parent=np.array([-1]), seg_len=np.array([0.0]), seg_diam=np.array([17.8]),
                      densities=_hh_densities(1, np.ones(1, dtype=bool)), cm=1.0, ra=30.0, v0=-65.0,
                      spike_thresh=-20.0)
    spec.cells.append(hh)
    spec.populations.append(Population("hh", "hhcell", n_hh))
    n = n_src + n_izh + n_hh
    post = np.repeat(np.arange(n_src, n), fan_in)
    pre = rng.integers(0, n, size=post.size)
    pre = np.where(pre == post, (pre + 1) % n, pre)
    delay = _round_us(rng.uniform(0.5, 4.0, size=post.size))
    w = np.round(rng.uniform(0.5, 3.0, size=post.size), 4)
    two = rng.random(post.size) < 0.6
    spec.projections.append(_flat_projection(spec, "proj_e2", pre[two], post[two], "syn_e2", w[two], delay[two]))
    spec.projections.append(_flat_projection(spec, "proj_e1", pre[~two], post[~two], "syn_e1", w[~two], delay[~two]))
    rec = np.sort(rng.choice(np.arange(n_src, n), size=min(n_recorded, n - n_src), replace=False))
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, int(g)), 0) for g in rec]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


# ---------------------------------------------------------------------------
def event_sets(n_inst: int = 3, ports=("zero", "one"), n_frames: int = 60, n_izh: int = 8, n_hh: int = 6,
               fan_in: int = 4, length_ms: float = 60.0, dt_ms: float = 0.025, seed: int = 1234,
               n_recorded: int = 6) -> NetworkSpec:
    """Spike events read from a file (EDEN's EdenEventSetReader, ascii_v0)
    driving izhikevich2007 and single-compartment HH cells, which also
    connect among themselves.  The frames are seeded, with timestamps on
    and next to step boundaries, a frame out of order (ignored), a negative
    timestamp (never applied) and a repeated source within a frame."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("event_sets", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=2.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("iz", "izRS", n_izh))
    hh = PhysicalCell(name="hhcell", seg_parent=np.array([-1]), seg_len=np.array([0.0]), seg_diam=np.array([17.8]),
                      densities=_hh_densities(1, np.ones(1, dtype=bool)), cm=1.0, ra=30.0, v0=-65.0,
                      spike_thresh=-20.0)
    spec.cells.append(hh)
    spec.populations.append(Population("hh", "hhcell", n_hh))
    n_cells = n_izh + n_hh
    times = np.sort(np.round(rng.uniform(0.0, length_ms * 1e-3, n_frames), 6))
    times[:4] = [0.0, 0.001, 0.0010001, 0.00099999]
    frames = []
    for t in np.sort(times):
        k = int(rng.integers(1, 4))
        pairs = [(int(rng.integers(0, n_inst)), int(rng.integers(0, len(ports)))) for _ in range(k)]
        frames.append((float(t), pairs))
    frames.insert(10, (frames[5][0], [(0, 0)]))            # not after the previous frame: ignored
    frames.insert(0, (-0.001, [(1, 1)]))                    # negative: never applied
    frames[20] = (frames[20][0], frames[20][1] + frames[20][1][:1])   # a source twice in one frame
    reader = EventSetReaderCell("evr", n_inst, list(ports), frames, href="evr_events.txt")
    spec.cells.append(reader)
    spec.populations.append(Population("evr", "evr", n_inst * len(ports)))
    n_src = n_inst * len(ports)
    post = np.repeat(np.arange(n_cells), fan_in)
    from_reader = rng.random(post.size) < 0.5
    pre = np.where(from_reader, n_cells + rng.integers(0, n_src, post.size), rng.integers(0, n_cells, post.size))
    pre = np.where(pre == post, (pre + 1) % n_cells, pre)
    delay = _round_us(rng.uniform(0.5, 3.0, size=post.size))
    w = np.round(rng.uniform(1.0, 4.0, size=post.size), 4)
    spec.projections.append(_flat_projection(spec, "proj_e2", pre, post, "syn_e2", w, delay))
    rec = np.sort(rng.choice(n_cells, size=min(n_recorded, n_cells), replace=False))
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, int(g)), 0) for g in rec]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n_cells)]
    return spec


# ---------------------------------------------------------------------------
def point_neurons(n_per_kind: int = 8, fan_in: int = 6, length_ms: float = 100.0, dt_ms: float = 0.025,
                  seed: int = 1234, n_recorded: int = 10) -> NetworkSpec:
    """One population of each of iafTauCell, iafTauRefCell, iafCell,
    iafRefCell and adExIaFCell (seeded parameters around the NeuroML
    examples'), a DC pulse into every cell that takes current and recurrent
    expTwo (excitatory) and expOne (inhibitory) synapses onto them; the Tau
    kinds take no input (they start at their leak reversal, above threshold,
    and fire periodically) but drive the others."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("point_neurons", dt_ms, length_ms, seed)
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=2.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    spec.synapses.append(SynapseType("syn_i1", SYN_EXPONE, gbase=2.0, erev=-80.0, tau_decay=3.0))
    r = lambda lo, hi: float(np.round(rng.uniform(lo, hi), 4))
    spec.cells.append(IafCell("iafTau", "iafTauCell", leak_reversal=-50.0, thresh=-55.0, reset=-70.0,
                              tau=r(20.0, 40.0)))
    spec.cells.append(IafCell("iafTauRef", "iafTauRefCell", leak_reversal=-50.0, thresh=-55.0, reset=-70.0,
                              tau=r(20.0, 40.0), refract=r(3.0, 7.0)))
    spec.cells.append(IafCell("iaf", "iafCell", leak_reversal=-70.0, thresh=-55.0, reset=-70.0, C=r(0.8, 1.2) * 1e3,
                              leak_conductance=r(40.0, 60.0)))
    spec.cells.append(IafCell("iafRef", "iafRefCell", leak_reversal=-70.0, thresh=-55.0, reset=-70.0,
                              C=r(0.8, 1.2) * 1e3, leak_conductance=r(40.0, 60.0), refract=r(3.0, 7.0)))
    spec.cells.append(AdExCell("adEx", C=281.0, gL=30.0, EL=-70.6, VT=-50.4, thresh=-40.4, reset=-48.5, delT=2.0,
                               tauw=40.0, refract=r(0.0, 1.0), a=4.0, b=0.08))
    for c in spec.cells:
        spec.populations.append(Population(f"p_{c.name}", c.name, n_per_kind))
    n = n_per_kind * len(spec.cells)
    driven = np.arange(2 * n_per_kind, n)          # the Tau kinds receive no current
    amp = np.round(rng.uniform(0.4, 1.2, len(driven)), 4)
    spec.pulses.append(PulseInputs("*", driven, np.zeros(len(driven), int), np.full(len(driven), 5.0),
                                   np.full(len(driven), length_ms - 20.0), amp))
    post = np.repeat(driven, fan_in)
    pre = rng.integers(0, n, size=post.size)
    pre = np.where(pre == post, (pre + 1) % n, pre)
    delay = _round_us(rng.uniform(0.5, 3.0, size=post.size))
    w = np.round(rng.uniform(0.5, 2.0, size=post.size), 4)
    exc = rng.random(post.size) < 0.75
    spec.projections.append(_flat_projection(spec, "proj_e2", pre[exc], post[exc], "syn_e2", w[exc], delay[exc]))
    spec.projections.append(_flat_projection(spec, "proj_i1", pre[~exc], post[~exc], "syn_i1", w[~exc], delay[~exc]))
    rec = np.sort(rng.choice(n, size=min(n_recorded, n), replace=False))
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, int(g)), 0) for g in rec]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


# ---------------------------------------------------------------------------
def timed_inputs(n_hh: int = 6, n_izh: int = 6, per_cell: int = 3, length_ms: float = 60.0, dt_ms: float = 0.025,
                 seed: int = 1234, n_recorded: int = 8) -> NetworkSpec:
    """timedSynapticInput spike lists (seeded times, some on and next to step
    boundaries, some before the first step and after the run) driving expTwo
    and expOne synapses on single-compartment HH and izhikevich2007 cells,
    which also connect among themselves."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("timed_inputs", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=3.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    spec.synapses.append(SynapseType("syn_e1", SYN_EXPONE, gbase=4.0, erev=0.0, tau_decay=2.0))
    hh = PhysicalCell(name="hhcell", seg_parent=np.array([-1]), seg_len=np.array([0.0]), seg_diam=np.array([17.8]),
                      densities=_hh_densities(1, np.ones(1, dtype=bool)), cm=1.0, ra=30.0, v0=-65.0,
                      spike_thresh=-20.0)
    spec.cells.append(hh)
    spec.populations.append(Population("hh", "hhcell", n_hh))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("iz", "izRS", n_izh))
    n = n_hh + n_izh
    for syn in ("syn_e2", "syn_e1"):
        cells = np.repeat(np.arange(n), per_cell)
        times = []
        for k in range(len(cells)):
            t = np.round(np.sort(rng.uniform(-2.0, length_ms + 5.0, size=rng.integers(2, 12))), 4)
            if k == 0:
                t = np.concatenate([t, [0.0, 10.0, 9.9999, 10.0001, 20.025, 20.0251]])
            times.append(t)
        spec.timed.append(TimedInputs(syn, cells, np.zeros(len(cells), np.int64), times,
                                      np.round(rng.uniform(0.5, 2.0, len(cells)), 4)))
    post = np.repeat(np.arange(n), 3)
    pre = rng.integers(0, n, size=post.size)
    pre = np.where(pre == post, (pre + 1) % n, pre)
    spec.projections.append(_flat_projection(spec, "proj_e2", pre, post, "syn_e2",
                                             np.round(rng.uniform(0.2, 1.0, post.size), 4),
                                             _round_us(rng.uniform(0.5, 3.0, size=post.size))))
    rec = np.sort(rng.choice(n, size=min(n_recorded, n), replace=False))
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, int(g)), 0) for g in rec]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


def input_kinds(n_mc: int = 6, n_izh: int = 4, length_ms: float = 80.0, dt_ms: float = 0.025,
                seed: int = 1234) -> NetworkSpec:
    """Every input kind on the same compartments: one branching cell type
    (HH soma, five passive dendrite segments) in two populations plus
    izhikevich2007 cells, with pulse, sine and ramp generators (weighted),
    several Poisson components (up to three on one soma, others on
    dendrites, so their random draws are numbered past the first), timed
    inputs on passive dendrites, and recurrent expTwo connections."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("input_kinds", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=2.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    spec.synapses.append(SynapseType("syn_e1", SYN_EXPONE, gbase=1.5, erev=0.0, tau_decay=3.0))
    parent = np.array([-1, 0, 1, 2, 1, 4])
    soma = np.zeros(len(parent), dtype=bool)
    soma[0] = True
    spec.cells.append(PhysicalCell("mc", parent, np.array([20.0, 60.0, 50.0, 40.0, 70.0, 30.0]),
                                   np.array([20.0, 2.0, 1.5, 1.0, 1.5, 1.0]),
                                   _hh_densities(len(parent), soma), cm=1.0, ra=150.0, v0=-65.0,
                                   spike_thresh=-20.0, seg_groups={"soma_group": soma, "dend_group": ~soma}))
    n_a = n_mc // 2
    spec.populations.append(Population("mcA", "mc", n_a))
    spec.populations.append(Population("mcB", "mc", n_mc - n_a))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("iz", "izRS", n_izh))
    mc = np.arange(n_mc)
    iz = n_mc + np.arange(n_izh)
    # weighted pulses (inputW) on two somata
    spec.pulses.append(PulseInputs("*", mc[:2], np.zeros(2, int), np.array([5.0, 30.0]), np.array([20.0, 40.0]),
                                   np.array([0.25, 0.4]), np.array([0.7, 1.3])))
    # sine generators: somata, a dendrite, izhikevich cells
    cells = np.concatenate([mc[:3], mc[3:5], iz[:2]])
    segs = np.concatenate([np.zeros(3, int), np.array([3, 5]), np.zeros(2, int)])
    n = len(cells)
    spec.waves.append(WaveInputs(WAVE_SINE, cells, segs, np.round(rng.uniform(0.0, 20.0, n), 3),
                                 np.round(rng.uniform(20.0, 60.0, n), 3),
                                 np.where(cells >= n_mc, 0.4, 0.3) * np.round(rng.uniform(0.5, 1.0, n), 3),
                                 np.round(rng.uniform(5.0, 25.0, n), 3), np.round(rng.uniform(-1.0, 1.0, n), 3),
                                 np.round(rng.uniform(0.5, 1.8, n), 3)))
    # ramp generators (baseline before and after the ramp)
    cells = np.concatenate([mc[2:5], iz[1:3]])
    segs = np.array([2, 0, 4, 0, 0])
    n = len(cells)
    scale = np.where(cells >= n_mc, 0.5, 0.3)
    spec.waves.append(WaveInputs(WAVE_RAMP, cells, segs, np.round(rng.uniform(0.0, 20.0, n), 3),
                                 np.round(rng.uniform(20.0, 50.0, n), 3),
                                 np.round(scale * rng.uniform(0.0, 0.5, n), 4),
                                 np.round(scale * rng.uniform(0.5, 1.0, n), 4),
                                 np.round(scale * rng.uniform(0.0, 0.2, n), 4),
                                 np.round(rng.uniform(0.5, 1.5, n), 3)))
    # Poisson components, in definition order: somata of every mc cell; a
    # second one on some somata and dendrites; a third on a dendrite and some
    # somata; two on the izhikevich cells
    spec.poissons.append(PoissonInputs("*", "syn_e2", 60.0, np.repeat(mc, 2), np.zeros(2 * n_mc, int)))
    spec.poissons.append(PoissonInputs("*", "syn_e1", 40.0, np.concatenate([mc[::2], mc[1::2]]),
                                       np.concatenate([np.zeros(len(mc[::2]), int), np.full(len(mc[1::2]), 2)])))
    spec.poissons.append(PoissonInputs("*", "syn_e2", 150.0, np.concatenate([mc, mc[:3]]),
                                       np.concatenate([np.full(n_mc, 4), np.zeros(3, int)])))
    spec.poissons.append(PoissonInputs("*", "syn_e1", 30.0, iz, np.zeros(n_izh, int)))
    spec.poissons.append(PoissonInputs("*", "syn_e2", 200.0, np.repeat(iz, 2), np.zeros(2 * n_izh, int)))
    # timed inputs on passive dendrite compartments
    times = [np.round(np.sort(rng.uniform(0.0, length_ms, rng.integers(3, 9))), 4) for _ in range(n_mc)]
    spec.timed.append(TimedInputs("syn_e2", mc, np.full(n_mc, 5), times, np.round(rng.uniform(0.5, 2.0, n_mc), 4)))
    # recurrent connections
    n_all = n_mc + n_izh
    post = np.repeat(np.arange(n_all), 2)
    pre = rng.integers(0, n_all, size=post.size)
    pre = np.where(pre == post, (pre + 1) % n_all, pre)
    post_seg = np.where(post < n_mc, rng.integers(0, len(parent), size=post.size), 0)
    spec.projections.append(_flat_projection(spec, "proj_e2", pre, post, "syn_e2",
                                             np.round(rng.uniform(0.2, 0.8, post.size), 4),
                                             _round_us(rng.uniform(0.5, 3.0, size=post.size)), post_seg=post_seg))
    cols = [(int(c), 0) for c in mc] + [(int(mc[1]), 2), (int(mc[3]), 3), (int(mc[4]), 5), (int(mc[0]), 4)]
    cols += [(int(c), 0) for c in iz]
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), seg) for g, seg in cols]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n_all)]
    return spec


def gate_kind_channels() -> list:
    """Leak plus sodium, delayed-rectifier and A-type potassium channels
    whose gates use each built-in gate kind and both q10 settings, and a
    persistent sodium channel with an instantaneous gate."""
    q10 = ("exp", 3.0, 6.3)
    leak = Channel("passiveChan")
    na = Channel("naT", [
        Gate("m", 3, Rate(RATE_EXPLINEAR, 1.0, -40.0, 10.0), Rate(RATE_EXP, 4.0, -65.0, -18.0), "ratesInf",
             inf=Rate(RATE_SIGMOID, 1.0, -40.0, 9.0), q10=q10),
        Gate("h", 1, kind="tauInf", tau=3.0, inf=Rate(RATE_SIGMOID, 1.0, -62.0, -7.0), q10=q10),
    ], species="na")
    kdr = Channel("kdr", [
        Gate("n", 4, Rate(RATE_EXPLINEAR, 0.1, -55.0, 10.0), Rate(RATE_EXP, 0.125, -65.0, -80.0), "ratesTau",
             tau=3.5, q10=("fixed", 1.5)),
    ], species="k")
    ka = Channel("kA", [
        Gate("a", 3, Rate(RATE_EXP, 0.2, -50.0, 20.0), Rate(RATE_SIGMOID, 0.3, -70.0, -10.0), "ratesTauInf",
             tau=2.0, inf=Rate(RATE_SIGMOID, 1.0, -45.0, 12.0), q10=q10),
        Gate("b", 1, Rate(RATE_EXP, 0.02, -80.0, -15.0), Rate(RATE_SIGMOID, 0.05, -60.0, 8.0), q10=q10),
    ], species="k")
    nap = Channel("naP", [Gate("m", 1, kind="instantaneous", inf=Rate(RATE_SIGMOID, 1.0, -52.0, 5.0))], species="na")
    return [leak, na, kdr, ka, nap]


def gate_kinds(n_single: int = 8, n_branch: int = 4, length_ms: float = 60.0, dt_ms: float = 0.025,
               seed: int = 1234, temperature: float = 16.3) -> NetworkSpec:
    """Cells whose channels use every built-in gate kind (gate_kind_channels)
    at 16.3 degC: single compartments with DC pulses of seeded amplitude and
    branching cells with the active channels on soma and first dendrite,
    Poisson drive and connections among all cells."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("gate_kinds", dt_ms, length_ms, seed, channels=gate_kind_channels())
    spec.temperature = temperature
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=3.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))

    def dens(n_seg, active):
        allseg = np.ones(n_seg, bool)
        return [ChannelDensity(0, 0.3, -54.387, allseg), ChannelDensity(1, 120.0, 50.0, active.copy()),
                ChannelDensity(2, 36.0, -77.0, active.copy()), ChannelDensity(3, 8.0, -77.0, active.copy()),
                ChannelDensity(4, 0.8, 50.0, active.copy())]

    one = np.ones(1, bool)
    spec.cells.append(PhysicalCell("single", np.array([-1]), np.array([0.0]), np.array([17.8]), dens(1, one),
                                   cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0))
    parent = np.array([-1, 0, 1, 1, 0])
    active = np.array([True, True, False, False, False])
    spec.cells.append(PhysicalCell("branch", parent, np.array([20.0, 40.0, 60.0, 60.0, 80.0]),
                                   np.array([20.0, 3.0, 1.5, 1.5, 2.0]), dens(len(parent), active), cm=1.0,
                                   ra=120.0, v0=-65.0, spike_thresh=-20.0,
                                   seg_groups={"soma_group": parent < 0, "dend_group": parent >= 0,
                                               "active_group": active}))
    spec.populations.append(Population("single", "single", n_single))
    spec.populations.append(Population("branch", "branch", n_branch))
    n = n_single + n_branch
    spec.pulses.append(PulseInputs("*", np.arange(n_single), np.zeros(n_single, int),
                                   np.round(rng.uniform(0.0, 10.0, n_single), 3), np.full(n_single, length_ms),
                                   np.round(rng.uniform(0.05, 0.35, n_single), 4)))
    br = n_single + np.arange(n_branch)
    spec.poissons.append(PoissonInputs("*", "syn_e2", 400.0, np.repeat(br, 4), np.tile([0, 0, 2, 4], n_branch)))
    post = np.repeat(np.arange(n), 2)
    pre = rng.integers(0, n, size=post.size)
    pre = np.where(pre == post, (pre + 1) % n, pre)
    spec.projections.append(_flat_projection(spec, "proj_e2", pre, post, "syn_e2",
                                             np.round(rng.uniform(0.1, 0.5, post.size), 4),
                                             _round_us(rng.uniform(0.5, 3.0, size=post.size))))
    cols = [(g, 0) for g in range(0, n_single, 2)] + [(int(br[0]), 0), (int(br[1]), 2), (int(br[2]), 4)]
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), seg) for g, seg in cols]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


def dl_inputs(n_dl: int = 6, length_ms: float = 100.0, dt_ms: float = 0.025, seed: int = 1234) -> NetworkSpec:
    """izhikevichCell instances (mixed-mode parameters) driven by
    pulseGeneratorDL, sineGeneratorDL and rampGeneratorDL inputs with seeded
    amplitudes, weighted, beside izhikevich2007 cells with pulse and sine
    generators; the two kinds connect through expOne synapses only into the
    izhikevich2007 cells.  Two fitzHughNagumoCell oscillators run beside
    them (no inputs)."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("dl_inputs", dt_ms, length_ms, seed)
    spec.cells.append(IzhikevichCell("izMixed", v0=-70.0, thresh=30.0, a=0.02, b=0.2, c=-55.0, d=4.0))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.synapses.append(SynapseType("syn_e1", SYN_EXPONE, gbase=2.0, erev=0.0, tau_decay=2.0))
    spec.cells.append(FitzHughNagumoCell("fn1", I=0.8))
    spec.populations += [Population("dl", "izMixed", n_dl), Population("iz", "izRS", 3), Population("fn", "fn1", 2)]
    dl = np.arange(n_dl)
    spec.pulses.append(PulseInputs("*", dl, np.zeros(n_dl, int), np.round(rng.uniform(0.0, 20.0, n_dl), 3),
                                   np.round(rng.uniform(30.0, 70.0, n_dl), 3), np.round(rng.uniform(5.0, 15.0, n_dl), 3),
                                   np.round(rng.uniform(0.6, 1.2, n_dl), 3), dimensionless=True))
    k = n_dl // 2
    one = lambda x: np.full(k, x)
    spec.waves.append(WaveInputs(WAVE_SINE, dl[:k], np.zeros(k, int), one(20.0), one(50.0),
                                 np.round(rng.uniform(10.0, 40.0, k), 3), one(10.0), one(1.0), np.ones(k),
                                 dimensionless=True))
    spec.waves.append(WaveInputs(WAVE_RAMP, dl[k:], np.zeros(n_dl - k, int), np.full(n_dl - k, 30.0),
                                 np.full(n_dl - k, 60.0), np.full(n_dl - k, -32.0), np.full(n_dl - k, 50.0),
                                 np.full(n_dl - k, -2.0), np.full(n_dl - k, 0.5), dimensionless=True))
    iz = n_dl + np.arange(3)
    spec.pulses.append(PulseInputs("*", iz, np.zeros(3, int), np.zeros(3), np.full(3, length_ms),
                                   np.array([0.08, 0.1, 0.12])))
    spec.projections.append(_flat_projection(spec, "proj_e1", dl[:3], iz, "syn_e1", np.full(3, 0.5),
                                             np.full(3, 1.0)))
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), 0) for g in range(n_dl + 5)]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n_dl + 3)]
    return spec


CUSTOM_SETUP_TEXT = """
# izhikevich2007Cell instances
set cell izh 1,3 all v0 -64 mV
set cell izh all all d multi pA
values 80 100 120 60 90 150
set cell izh 2,4 all a 0.05 per_ms
set cell izh 5 all vpeak 30 mV
# iafRefCell instances
set cell iaf 0,2 all thresh -52 mV
set cell iaf all all refract multi ms
values 2 4 6 8
# adExIaFCell instances
set cell adex 1 all b 0.1 nA
set cell adex all all EL multi mV
values -70.6 -68 -72 -66
set cell izh 3 all v0 -58 mV
"""


def custom_setup(length_ms: float = 100.0, dt_ms: float = 0.025, seed: int = 1234) -> NetworkSpec:
    """Point-neuron populations whose parameters an EdenCustomSetup file
    overrides per instance (single values, per-instance lists, repeated
    statements on the same instance), driven by DC pulses from one input
    list per population whose amplitudes, delays and durations the file
    sets per input."""
    from .custom_setup import parse
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("custom_setup", dt_ms, length_ms, seed)
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.cells.append(IafCell("iafRef", "iafRefCell", leak_reversal=-65.0, thresh=-50.0, reset=-65.0, C=200.0,
                              leak_conductance=10.0, refract=3.0))
    spec.cells.append(AdExCell("adex", C=281.0, gL=30.0, EL=-70.6, VT=-50.4, thresh=-40.4, reset=-70.6, delT=2.0,
                               tauw=144.0, refract=0.0, a=4.0, b=0.0805))
    spec.populations += [Population("izh", "izRS", 6), Population("iaf", "iafRef", 4), Population("adex", "adex", 4)]
    n = 14
    # one input list per population, one pulse component each; the setup
    # file varies their amplitudes and timing per input
    sizes = {"stim_izh": (0, 6, 0.2), "stim_iaf": (6, 4, 0.3), "stim_adex": (10, 4, 0.8)}
    for lst, (g0, k, a) in sizes.items():
        spec.pulses.append(PulseInputs("*", g0 + np.arange(k), np.zeros(k, int), np.full(k, 5.0),
                                       np.full(k, length_ms), np.full(k, a),
                                       list_ids=[(lst, j) for j in range(k)]))
    text = CUSTOM_SETUP_TEXT + "".join([
        "set input stim_izh all amplitude multi nA\n",
        "values " + " ".join(str(x) for x in np.round(rng.uniform(0.1, 0.3, 6), 4)) + "\n",
        "set input stim_iaf 1,3 delay 20 ms\n",
        "set input stim_adex all duration multi ms\n",
        "values 30 50 70 90\n",
        "set input stim_adex 2 amplitude 1.0 nA\n"])
    spec.custom_setup = parse(text, spec)
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), 0) for g in range(n)]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


def random_sources(n_each: int = 4, n_izh: int = 8, n_hh: int = 6, fan_out: int = 3, length_ms: float = 100.0,
                   dt_ms: float = 0.025, seed: int = 1234) -> NetworkSpec:
    """Random spike generators (uniform intervals, Poisson, Poisson with a
    refractory floor), several instances each, so their per-cell seeds
    differ, connected to izhikevich and single-compartment HH cells through
    expOne synapses."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("random_sources", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses.append(SynapseType("syn_e1", SYN_EXPONE, gbase=6.0, erev=0.0, tau_decay=2.0))
    spec.cells += [SpikeGeneratorRandomCell("rnd", 3.0, 9.0), SpikeGeneratorPoissonCell("poi", 150.0),
                   SpikeGeneratorPoissonCell("refpoi", 120.0, 4.0),
                   Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0),
                   PhysicalCell("hhcell", np.array([-1]), np.array([0.0]), np.array([17.8]),
                                _hh_densities(1, np.ones(1, bool)), cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0)]
    for name in ("rnd", "poi", "refpoi"):
        spec.populations.append(Population(name, name, n_each))
    spec.populations.append(Population("iz", "izRS", n_izh))
    spec.populations.append(Population("hh", "hhcell", n_hh))
    n_src = 3 * n_each
    targets = n_src + np.arange(n_izh + n_hh)
    pre = np.repeat(np.arange(n_src), fan_out)
    post = rng.choice(targets, size=pre.size)
    spec.projections.append(_flat_projection(spec, "proj_e1", pre, post, "syn_e1",
                                             np.round(rng.uniform(0.3, 1.0, pre.size), 4),
                                             _round_us(rng.uniform(0.5, 2.0, size=pre.size))))
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, int(g)), 0) for g in targets[::3]]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n_src + n_izh + n_hh)]
    return spec


def voltage_clamps(n_hh: int = 4, n_branch: int = 2, n_izh: int = 2, length_ms: float = 60.0,
                   dt_ms: float = 0.025, seed: int = 1234) -> NetworkSpec:
    """voltageClamp (one target between delay and delay + duration) and
    voltageClampTriple (conditioning, testing and return targets) on HH
    somata, a passive dendrite and izhikevich cells, series resistances
    10-100 MOhm, weighted; DC pulses make the cells fire outside the
    clamped phases."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("voltage_clamps", dt_ms, length_ms, seed, channels=hh_channels())
    spec.cells.append(PhysicalCell("hhcell", np.array([-1]), np.array([0.0]), np.array([17.8]),
                                   _hh_densities(1, np.ones(1, bool)), cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0))
    parent = np.array([-1, 0, 1])
    soma = parent < 0
    spec.cells.append(PhysicalCell("branch", parent, np.array([20.0, 80.0, 60.0]), np.array([20.0, 2.0, 1.5]),
                                   _hh_densities(3, soma), cm=1.0, ra=150.0, v0=-65.0, spike_thresh=-20.0,
                                   seg_groups={"soma_group": soma, "dend_group": ~soma}))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("hh", "hhcell", n_hh))
    spec.populations.append(Population("branch", "branch", n_branch))
    spec.populations.append(Population("iz", "izRS", n_izh))
    n = n_hh + n_branch + n_izh
    spec.pulses.append(PulseInputs("*", np.arange(n), np.zeros(n, int), np.zeros(n), np.full(n, length_ms),
                                   np.round(rng.uniform(0.05, 0.3, n), 4)))
    br = n_hh + np.arange(n_branch)
    iz = n_hh + n_branch + np.arange(n_izh)
    cells = np.concatenate([np.arange(n_hh), br, iz])
    segs = np.concatenate([np.zeros(n_hh, int), np.full(n_branch, 2), np.zeros(n_izh, int)])
    k = len(cells)
    spec.clamps.append(ClampInputs(False, cells, segs, np.round(rng.uniform(5.0, 20.0, k), 3),
                                   np.round(rng.uniform(10.0, 25.0, k), 3), np.full(k, np.nan),
                                   np.round(rng.uniform(-80.0, -40.0, k), 2), np.full(k, np.nan),
                                   np.round(rng.uniform(10.0, 100.0, k), 2), np.round(rng.uniform(0.5, 1.5, k), 3)))
    spec.clamps.append(ClampInputs(True, br, np.zeros(n_branch, int), np.full(n_branch, 15.0),
                                   np.full(n_branch, 20.0), np.array([-63.77, -70.0]), np.array([-30.0, -45.0]),
                                   np.array([-40.77, -55.0]), np.array([50.0, 80.0]), np.ones(n_branch)))
    cols = [(g, 0) for g in range(n)] + [(int(br[0]), 2)]
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), seg) for g, seg in cols]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


def alpha_synapses(n_hh: int = 6, n_izh: int = 6, n_branch: int = 3, length_ms: float = 80.0, dt_ms: float = 0.025,
                   seed: int = 1234) -> NetworkSpec:
    """alphaSynapse (conductance) and alphaCurrentSynapse (current) on
    single-compartment HH cells, the dendrites of branching cells and
    izhikevich2007 cells: recurrent connections of both kinds, Poisson
    inputs driving each kind, and timed inputs (some in the same steps as
    other events), beside an expTwo connection onto the same compartments."""
    from .network import SYN_ALPHA, SYN_ALPHA_CURRENT
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("alpha_synapses", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses.append(SynapseType("syn_alpha", SYN_ALPHA, gbase=2.0, erev=0.0, tau_decay=2.0))
    spec.synapses.append(SynapseType("syn_alpha_i", SYN_ALPHA_CURRENT, gbase=0.08, erev=0.0, tau_decay=3.0))
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=1.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    spec.cells.append(PhysicalCell("hhcell", np.array([-1]), np.array([0.0]), np.array([17.8]),
                                   _hh_densities(1, np.ones(1, bool)), cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0))
    parent = np.array([-1, 0, 1])
    soma = parent < 0
    spec.cells.append(PhysicalCell("branch", parent, np.array([20.0, 60.0, 50.0]), np.array([20.0, 2.0, 1.5]),
                                   _hh_densities(3, soma), cm=1.0, ra=150.0, v0=-65.0, spike_thresh=-20.0,
                                   seg_groups={"soma_group": soma, "dend_group": ~soma}))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("hh", "hhcell", n_hh))
    spec.populations.append(Population("branch", "branch", n_branch))
    spec.populations.append(Population("iz", "izRS", n_izh))
    hh = np.arange(n_hh)
    br = n_hh + np.arange(n_branch)
    iz = n_hh + n_branch + np.arange(n_izh)
    n = n_hh + n_branch + n_izh
    # a DC drive on a third of the cells
    drv = np.arange(0, n, 3)
    amp = np.where(drv >= n_hh + n_branch, 0.12, 0.12)
    spec.pulses.append(PulseInputs("*", drv, np.zeros(len(drv), int), np.full(len(drv), 2.0),
                                   np.full(len(drv), length_ms), np.round(amp * rng.uniform(0.8, 1.6, len(drv)), 4)))
    # recurrent connections of each kind, somata and dendrites
    for syn in ("syn_alpha", "syn_alpha_i", "syn_e2"):
        post = np.repeat(np.arange(n), 2)
        pre = rng.integers(0, n, size=post.size)
        pre = np.where(pre == post, (pre + 1) % n, pre)
        seg = np.where((post >= n_hh) & (post < n_hh + n_branch), rng.integers(0, 3, size=post.size), 0)
        spec.projections.append(_flat_projection(spec, f"proj_{syn}", pre, post, syn,
                                                 np.round(rng.uniform(0.5, 1.5, post.size), 4),
                                                 _round_us(rng.uniform(0.5, 3.0, size=post.size)), post_seg=seg))
    # Poisson inputs of both alpha kinds
    spec.poissons.append(PoissonInputs("*", "syn_alpha", 60.0, np.concatenate([hh, br, iz]),
                                       np.concatenate([np.zeros(n_hh, int), np.full(n_branch, 2), np.zeros(n_izh, int)])))
    spec.poissons.append(PoissonInputs("*", "syn_alpha_i", 80.0, np.concatenate([hh, iz]),
                                       np.zeros(n_hh + n_izh, int)))
    # timed inputs of both alpha kinds
    for syn in ("syn_alpha", "syn_alpha_i"):
        cells = np.concatenate([hh[::2], iz[::2]])
        times = [np.round(np.sort(rng.uniform(0.0, length_ms, rng.integers(3, 9))), 4) for _ in cells]
        times[0] = np.concatenate([times[0], [10.0, 10.0001, 20.025]])
        spec.timed.append(TimedInputs(syn, cells, np.zeros(len(cells), np.int64), times,
                                      np.round(rng.uniform(0.5, 1.5, len(cells)), 4)))
    cols = [(g, 0) for g in range(n)] + [(int(b), 2) for b in br]
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), seg) for g, seg in cols]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


def pynn_synapses(n_hh: int = 6, n_branch: int = 3, n_izh: int = 4, length_ms: float = 80.0, dt_ms: float = 0.025,
                  seed: int = 4321) -> NetworkSpec:
    """The PyNN synapses (expCondSynapse, alphaCondSynapse, expCurrSynapse,
    alphaCurrSynapse) and expThreeSynapse on single-compartment HH cells,
    the dendrites of branching cells and izhikevich2007 cells: recurrent
    connections of each kind, Poisson inputs of three PyNN kinds and timed
    inputs of four kinds (some in the same steps as other events)."""
    from .network import SYN_ALPHA, SYN_ALPHA_CURRENT, SYN_EXPONE_CURRENT, SYN_EXPTHREE
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("pynn_synapses", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses += [
        SynapseType("syn_expcond", SYN_EXPONE, 1000.0, 0.0, 2.0, form="expCondSynapse"),
        SynapseType("syn_alphacond", SYN_ALPHA, 1000.0, -10.0, 1.5, form="alphaCondSynapse"),
        SynapseType("syn_expcurr", SYN_EXPONE_CURRENT, 1.0, 0.0, 3.0, form="expCurrSynapse"),
        SynapseType("syn_alphacurr", SYN_ALPHA_CURRENT, 1.0, 0.0, 2.5, form="alphaCurrSynapse"),
        SynapseType("syn_e3", SYN_EXPTHREE, 1.5, 0.0, 1.5, tau_rise=0.5, gbase2=0.8, tau_decay2=5.0),
    ]
    # PyNN weights are the state's jump: uS for the conductance kinds, nA
    # for the current kinds
    wscale = {"syn_expcond": 0.002, "syn_alphacond": 0.002, "syn_expcurr": 0.1, "syn_alphacurr": 0.05, "syn_e3": 1.0}
    spec.cells.append(PhysicalCell("hhcell", np.array([-1]), np.array([0.0]), np.array([17.8]),
                                   _hh_densities(1, np.ones(1, bool)), cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0))
    parent = np.array([-1, 0, 1, 1])
    soma = parent < 0
    spec.cells.append(PhysicalCell("branch", parent, np.array([20.0, 60.0, 50.0, 40.0]),
                                   np.array([20.0, 2.0, 1.5, 1.2]), _hh_densities(4, soma), cm=1.0, ra=150.0,
                                   v0=-65.0, spike_thresh=-20.0, seg_groups={"soma_group": soma, "dend_group": ~soma}))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("hh", "hhcell", n_hh))
    spec.populations.append(Population("branch", "branch", n_branch))
    spec.populations.append(Population("iz", "izRS", n_izh))
    hh = np.arange(n_hh)
    br = n_hh + np.arange(n_branch)
    iz = n_hh + n_branch + np.arange(n_izh)
    n = n_hh + n_branch + n_izh
    drv = np.arange(0, n, 3)
    spec.pulses.append(PulseInputs("*", drv, np.zeros(len(drv), int), np.full(len(drv), 2.0),
                                   np.full(len(drv), length_ms), np.round(0.12 * rng.uniform(0.8, 1.6, len(drv)), 4)))
    for syn in ("syn_expcond", "syn_alphacond", "syn_expcurr", "syn_alphacurr", "syn_e3"):
        post = np.repeat(np.arange(n), 2)
        pre = rng.integers(0, n, size=post.size)
        pre = np.where(pre == post, (pre + 1) % n, pre)
        seg = np.where((post >= n_hh) & (post < n_hh + n_branch), rng.integers(0, 4, size=post.size), 0)
        spec.projections.append(_flat_projection(spec, f"proj_{syn}", pre, post, syn,
                                                 np.round(wscale[syn] * rng.uniform(0.5, 1.5, post.size), 5),
                                                 _round_us(rng.uniform(0.5, 3.0, size=post.size)), post_seg=seg))
    # (a Poisson input's weight is 1: on an expCondSynapse that is a 1 uS
    # jump, left out)
    for syn, rate in (("syn_alphacond", 40.0), ("syn_expcurr", 80.0), ("syn_alphacurr", 50.0)):
        cells = np.concatenate([hh, br, iz])
        segs = np.concatenate([np.zeros(n_hh, int), np.full(n_branch, 3), np.zeros(n_izh, int)])
        spec.poissons.append(PoissonInputs("*", syn, rate, cells, segs))
    for syn in ("syn_expcond", "syn_expcurr", "syn_alphacurr", "syn_e3"):
        cells = np.concatenate([hh[::2], iz[::2]])
        times = [np.round(np.sort(rng.uniform(0.0, length_ms, rng.integers(3, 9))), 4) for _ in cells]
        times[0] = np.concatenate([times[0], [10.0, 10.0001, 20.025]])
        spec.timed.append(TimedInputs(syn, cells, np.zeros(len(cells), np.int64), times,
                                      np.round(wscale[syn] * rng.uniform(0.5, 1.5, len(cells)), 5)))
    cols = [(g, 0) for g in range(n)] + [(int(b), 3) for b in br]
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), seg) for g, seg in cols]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


def continuous_synapses(n_pairs: int = 6, length_ms: float = 60.0, dt_ms: float = 0.01,
                        seed: int = 1234) -> NetworkSpec:
    """Continuous connections between HH cells (spiking under DC pulses)
    and the somata or dendrites of branching cells: linearGradedSynapse on
    either end with silentSynapse on the other, silentSynapse to
    gradedSynapse, gradedSynapse on both ends, a linearGradedSynapse on an
    electrical connection, and a gapJunction on a continuous connection;
    weights 0.5-1.5.  (dt 0.01 ms: forward Euler on a graded synapse's s
    is stable while dt k / (1 - inf) < 2, which the reference's own test
    network keeps with dt 0.002 ms and k 0.025 per ms.)"""
    from .network import ContinuousProjection
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("continuous_synapses", dt_ms, length_ms, seed, channels=hh_channels())
    spec.gap_types += [GapJunctionType("lin", 2.0, kind="linearGradedSynapse"),
                       GapJunctionType("silent", 0.0, kind="silentSynapse"),
                       GapJunctionType("graded", 5.0, kind="gradedSynapse", delta=5.0, k=0.025, vth=-35.0, erev=0.0),
                       GapJunctionType("graded_inh", 3.0, kind="gradedSynapse", delta=4.0, k=0.02, vth=-40.0,
                                       erev=-80.0),
                       GapJunctionType("gap", 1.0)]
    spec.cells.append(PhysicalCell("hhcell", np.array([-1]), np.array([0.0]), np.array([17.8]),
                                   _hh_densities(1, np.ones(1, bool)), cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0))
    parent = np.array([-1, 0, 1])
    soma = parent < 0
    spec.cells.append(PhysicalCell("branch", parent, np.array([20.0, 60.0, 50.0]), np.array([20.0, 2.0, 1.5]),
                                   _hh_densities(3, soma), cm=1.0, ra=150.0, v0=-65.0, spike_thresh=-20.0,
                                   seg_groups={"soma_group": soma, "dend_group": ~soma}))
    spec.populations.append(Population("pre", "hhcell", n_pairs))
    spec.populations.append(Population("post", "branch", n_pairs))
    pre = np.arange(n_pairs)
    post = n_pairs + np.arange(n_pairs)
    spec.pulses.append(PulseInputs("*", pre, np.zeros(n_pairs, int), np.round(rng.uniform(2.0, 8.0, n_pairs), 3),
                                   np.full(n_pairs, 40.0), np.round(rng.uniform(0.1, 0.3, n_pairs), 4)))
    w = lambda n: np.round(rng.uniform(0.5, 1.5, n), 4)
    z = lambda n: np.zeros(n, np.int64)
    forms = [("lin", "silent"), ("silent", "lin"), ("silent", "graded"), ("graded", "graded_inh"),
             ("gap", "silent"), ("silent", "graded_inh")]
    for k, (ca, cb) in enumerate(forms):
        i = np.array([k % n_pairs, (k + 2) % n_pairs])
        seg = np.array([0, 2])
        spec.continuous.append(ContinuousProjection(f"cont_{k}", ca, cb, pre[i], z(2), post[i], seg, w(2)))
    spec.electrical.append(ElectricalProjection("lin_el", "lin", pre[[1, 4]], z(2), post[[3, 5]], np.array([1, 2]),
                                                w(2)))
    cols = [(int(g), 0) for g in pre] + [(int(g), seg) for g in post for seg in (0, 2)]
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), seg) for g, seg in cols]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, int(g)), 0) for g in np.concatenate([pre, post])]
    return spec


def gap_junctions(n_hh: int = 10, n_branch: int = 4, n_izh: int = 2, length_ms: float = 80.0,
                  dt_ms: float = 0.025, seed: int = 1234) -> NetworkSpec:
    """Gap junctions (two gapJunction types, 1 and 4 nS, weights 0.5-1.5)
    joining HH somata in a ring with random chords and HH somata to the
    passive dendrites of branching cells; DC pulses drive a third of the
    somata, so the rest are driven through the junctions, and expTwo
    synapses from the HH cells land on coupled compartments and on
    izhikevich cells."""
    rng = np.random.default_rng(seed)
    spec = NetworkSpec("gap_junctions", dt_ms, length_ms, seed, channels=hh_channels())
    spec.synapses.append(SynapseType("syn_e2", SYN_EXPTWO, gbase=1.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    spec.gap_types.append(GapJunctionType("gap_weak", 1.0))
    spec.gap_types.append(GapJunctionType("gap_strong", 4.0))
    spec.cells.append(PhysicalCell("hhcell", np.array([-1]), np.array([0.0]), np.array([17.8]),
                                   _hh_densities(1, np.ones(1, bool)), cm=1.0, ra=30.0, v0=-65.0, spike_thresh=-20.0))
    parent = np.array([-1, 0, 1, 0])
    soma = parent < 0
    spec.cells.append(PhysicalCell("branch", parent, np.array([20.0, 80.0, 60.0, 70.0]),
                                   np.array([20.0, 2.0, 1.5, 1.8]), _hh_densities(len(parent), soma), cm=1.0,
                                   ra=150.0, v0=-65.0, spike_thresh=-20.0,
                                   seg_groups={"soma_group": soma, "dend_group": ~soma}))
    spec.cells.append(Izhikevich2007Cell("izRS", a=0.03, d=100.0, c=-50.0))
    spec.populations.append(Population("hh", "hhcell", n_hh))
    spec.populations.append(Population("branch", "branch", n_branch))
    spec.populations.append(Population("iz", "izRS", n_izh))
    hh = np.arange(n_hh)
    br = n_hh + np.arange(n_branch)
    iz = n_hh + n_branch + np.arange(n_izh)
    driven = hh[::3]
    spec.pulses.append(PulseInputs("*", driven, np.zeros(len(driven), int),
                                   np.round(rng.uniform(2.0, 10.0, len(driven)), 3), np.full(len(driven), length_ms),
                                   np.round(rng.uniform(0.1, 0.3, len(driven)), 4)))
    spec.pulses.append(PulseInputs("*", iz, np.zeros(n_izh, int), np.zeros(n_izh), np.full(n_izh, length_ms),
                                   np.full(n_izh, 0.1)))
    # weak junctions: a ring of somata plus random chords
    pre = np.concatenate([hh, rng.choice(hh, n_hh // 2)])
    post = np.concatenate([np.roll(hh, -1), rng.choice(hh, n_hh // 2)])
    post = np.where(pre == post, (post + 1) % n_hh, post)
    spec.electrical.append(ElectricalProjection("gap_weak", "gap_weak", pre, np.zeros(len(pre), int), post,
                                                np.zeros(len(pre), int),
                                                np.round(rng.uniform(0.5, 1.5, len(pre)), 4)))
    # strong junctions: somata to the dendrites of the branching cells
    pre = rng.choice(hh, 2 * n_branch)
    post = np.repeat(br, 2)
    post_seg = np.tile([2, 3], n_branch)
    spec.electrical.append(ElectricalProjection("gap_strong", "gap_strong", pre, np.zeros(len(pre), int), post,
                                                post_seg, np.round(rng.uniform(0.5, 1.5, len(pre)), 4)))
    # chemical synapses onto coupled somata and dendrites, and izhikevich cells
    post = np.concatenate([hh[1::3], br, iz])
    pre = rng.choice(driven, len(post))
    post_seg = np.concatenate([np.zeros(len(hh[1::3]), int), np.full(n_branch, 2), np.zeros(n_izh, int)])
    spec.projections.append(_flat_projection(spec, "proj_e2", pre, post, "syn_e2",
                                             np.round(rng.uniform(0.5, 1.5, len(post)), 4),
                                             _round_us(rng.uniform(0.5, 3.0, len(post))), post_seg=post_seg))
    n = n_hh + n_branch + n_izh
    cols = [(g, 0) for g in range(n)] + [(int(b), 2) for b in br] + [(int(br[0]), 3)]
    spec.trace_columns = [OutputColumn(*_gid_to_pop(spec, g), seg) for g, seg in cols]
    spec.event_selections = [EventSelection(*_gid_to_pop(spec, g), 0) for g in range(n)]
    return spec


CONFIGS = {
    "single_comp_hh": single_comp_hh,
    "multicomp_net": multicomp_net,
    "izh_net": izh_net,
    "ball_and_stick": ball_and_stick,
    "mixed_scale": mixed_scale,
    "spike_sources": spike_sources,
    "event_sets": event_sets,
    "point_neurons": point_neurons,
    "timed_inputs": timed_inputs,
    "input_kinds": input_kinds,
    "gate_kinds": gate_kinds,
    "voltage_clamps": voltage_clamps,
    "gap_junctions": gap_junctions,
    "alpha_synapses": alpha_synapses,
    "pynn_synapses": pynn_synapses,
    "continuous_synapses": continuous_synapses,
    "routing_probe": routing_probe,
    "random_sources": random_sources,
    "custom_setup": custom_setup,
    "dl_inputs": dl_inputs,
}
