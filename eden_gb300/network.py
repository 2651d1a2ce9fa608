"""Neutral description of the NeuroML networks this path simulates.

A `NetworkSpec` holds, in numpy arrays, exactly the NeuroML content the
GPU path supports: physical (multi-compartment) cells with ionChannelHH
channels, izhikevich2007Cell point neurons, expOneSynapse / expTwoSynapse
synapses reached through `connectionWD` projections, pulseGenerator,
sineGenerator, rampGenerator, poissonFiringSynapse and timedSynapticInput
inputs, and the LEMS
`<Simulation>` with its `OutputFile` / `EventOutputFile` recorders.

Three producers/consumers share it:
  * workloads.py builds it from a seed (the synthetic configurations);
  * neuroml_io.py writes it as LEMS/NeuroML and reads it back from such files
    (the reference's input format, so the reference simulator can run the
    same model);
  * lowering.py turns it into the device-side structure-of-arrays model.

Quantities are stored in NeuroML's physiological units as written in the
XML (mV, ms, um, nS, nA, pF, mS/cm2, uF/cm2, ohm*cm, Hz) so that writing
and re-reading a spec is lossless; the conversion to engine units
(us, mV, nA, pF, uS, Mohm, um — eden/NeuroML.cpp:307-400) happens in
lowering.py.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


# ---------------------------------------------------------------------------
# Channel kinetics (ionChannelHH with gateHHrates, eden/NeuroML.cpp:4030-4110)
# ---------------------------------------------------------------------------
RATE_EXP = 0        # HHExpRate:        r * exp((v - mid) / s)
RATE_EXPLINEAR = 1  # HHExpLinearRate:  r * x / (1 - exp(-x)), x = (v - mid) / s
RATE_SIGMOID = 2    # HHSigmoidRate:    r / (1 + exp((mid - v) / s))

RATE_TYPE_NAMES = {RATE_EXP: "HHExpRate", RATE_EXPLINEAR: "HHExpLinearRate",
                   RATE_SIGMOID: "HHSigmoidRate"}


@dataclass
class Rate:
    kind: int
    rate: float      # per_ms
    midpoint: float  # mV
    scale: float     # mV


@dataclass
class Gate:
    """An HH gate.  `kind` is "rates" (gateHHrates), "tauInf", "ratesTau",
    "ratesInf", "ratesTauInf" or "instantaneous"; `tau` a fixedTimeCourse (ms) and `inf` an
    HH*Variable steady state (dimensionless rate) where the kind has them;
    `q10` None, ("fixed", factor) or ("exp", q10Factor, experimentalTemp
    degC)."""
    name: str
    instances: int
    forward: Optional[Rate] = None
    reverse: Optional[Rate] = None
    kind: str = "rates"
    tau: Optional[float] = None
    inf: Optional[Rate] = None
    q10: Optional[tuple] = None


@dataclass
class Channel:
    name: str
    gates: List[Gate] = field(default_factory=list)
    species: Optional[str] = None


def hh_channels() -> List[Channel]:
    """The classic squid-axon HH set (leak, Na m3h, K n4), with the rate
    constants of the reference example examples/NML2_SingleCompHHCell.nml."""
    leak = Channel("passiveChan")
    na = Channel("naChan", [
        Gate("m", 3, Rate(RATE_EXPLINEAR, 1.0, -40.0, 10.0), Rate(RATE_EXP, 4.0, -65.0, -18.0)),
        Gate("h", 1, Rate(RATE_EXP, 0.07, -65.0, -20.0), Rate(RATE_SIGMOID, 1.0, -35.0, 10.0)),
    ], species="na")
    k = Channel("kChan", [
        Gate("n", 4, Rate(RATE_EXPLINEAR, 0.1, -55.0, 10.0), Rate(RATE_EXP, 0.125, -65.0, -80.0)),
    ], species="k")
    return [leak, na, k]


# ---------------------------------------------------------------------------
# Cell types
# ---------------------------------------------------------------------------
@dataclass
class ChannelDensity:
    """channelDensity: `channel` (index into NetworkSpec.channels) on the
    segments whose mask is set, conductivity `cond` mS/cm2, reversal mV;
    `name` is its id, which paths to its gates' states use."""
    channel: int
    cond: float
    erev: float
    seg_mask: np.ndarray  # bool per segment
    name: str = ""


@dataclass
class PhysicalCell:
    """A NeuroML <cell>: an unbranched-or-branched tree of segments, one
    compartment per segment.

    seg_parent[i] < i (root = segment 0 with parent -1).  Segment i runs from
    its parent's distal point along +x by seg_len[i] um, a frustum from
    diameter seg_dprox[i] (proximal; None: seg_diam throughout, a cylinder)
    to seg_diam[i] um (distal); a zero-length root is a sphere of its distal
    diameter.
    """
    name: str
    seg_parent: np.ndarray
    seg_len: np.ndarray
    seg_diam: np.ndarray
    densities: List[ChannelDensity]
    cm: float = 1.0            # uF/cm2
    ra: float = 30.0           # ohm*cm
    v0: float = -65.0          # mV
    spike_thresh: float = -20.0  # mV
    seg_groups: dict = field(default_factory=dict)  # name -> bool mask (for writing)
    seg_dprox: Optional[np.ndarray] = None  # proximal diameters, um

    @property
    def n_seg(self) -> int:
        return int(len(self.seg_parent))


@dataclass
class Izhikevich2007Cell:
    name: str
    C: float = 100.0      # pF
    k: float = 0.7        # nS/mV
    vr: float = -60.0     # mV
    vt: float = -40.0     # mV
    vpeak: float = 35.0   # mV
    a: float = 0.03       # per_ms
    b: float = -2.0       # nS
    c: float = -50.0      # mV
    d: float = 100.0      # pA
    v0: float = -60.0     # mV


@dataclass
class IzhikevichCell:
    """izhikevichCell (the dimensionless form): v0, thresh mV; a, b, c, d
    dimensionless.  Its input current is dimensionless: it takes the
    *GeneratorDL inputs only."""
    name: str
    v0: float
    thresh: float
    a: float
    b: float
    c: float
    d: float


@dataclass
class FitzHughNagumoCell:
    """fitzHughNagumoCell: dimensionless V and W driven by the constant I;
    takes no input current and emits no spikes (its V is recorded as "V")."""
    name: str
    I: float


@dataclass
class IafCell:
    """iafTauCell, iafTauRefCell, iafCell or iafRefCell (`kind`), NeuroML
    units: mV, ms, nS, pF.  The *Tau* kinds have no capacitance, leak
    conductance or synaptic input; the *Ref* kinds a refractory period."""
    name: str
    kind: str                  # "iafTauCell", "iafTauRefCell", "iafCell", "iafRefCell"
    leak_reversal: float
    thresh: float
    reset: float
    tau: float = 0.0           # ms (Tau kinds)
    C: float = 0.0             # pF (iafCell, iafRefCell)
    leak_conductance: float = 0.0   # nS
    refract: float = 0.0       # ms (Ref kinds)


@dataclass
class AdExCell:
    """adExIaFCell (Brette and Gerstner 2005), NeuroML units: pF, nS, mV, ms, nA."""
    name: str
    C: float
    gL: float
    EL: float
    VT: float
    thresh: float
    reset: float
    delT: float
    tauw: float
    refract: float
    a: float
    b: float


@dataclass
class SpikeArrayCell:
    """spikeArray: a spike source with no membrane that emits spikes at the
    listed times (ms); a step emits at most one spike."""
    name: str
    times: np.ndarray


@dataclass
class SpikeGeneratorCell:
    """spikeGenerator: a spike source emitting every `period` ms, the first
    one period after t = 0."""
    name: str
    period: float


@dataclass
class SpikeGeneratorRandomCell:
    """spikeGeneratorRandom: intervals uniform in [min_isi, max_isi) ms."""
    name: str
    min_isi: float
    max_isi: float


@dataclass
class SpikeGeneratorPoissonCell:
    """spikeGeneratorPoisson (`min_isi` None) or spikeGeneratorRefPoisson
    (`min_isi` ms, a refractory floor on the intervals) at `rate` Hz."""
    name: str
    rate: float
    min_isi: Optional[float] = None


@dataclass
class EventSetReaderCell:
    """EdenEventSetReader: spike events streamed from a file, one source per
    (instance, port); `frames` are the file's lines in order, each a
    timestamp (s) and the (instance, port) pairs it names.  A population of
    instances * len(ports) sources, source instance * len(ports) + port."""
    name: str
    instances: int
    ports: list
    frames: list
    href: str = "events.txt"


SPIKE_SOURCE_TYPES = (SpikeArrayCell, SpikeGeneratorCell, EventSetReaderCell, SpikeGeneratorRandomCell,
                      SpikeGeneratorPoissonCell)


# ---------------------------------------------------------------------------
# Synapses and inputs
# ---------------------------------------------------------------------------
SYN_EXPONE = 0
SYN_EXPTWO = 1
SYN_ALPHA = 2           # alphaSynapse: conductance, rise and decay both tau
SYN_ALPHA_CURRENT = 3   # alphaCurrentSynapse: current ibase, rise and decay both tau
SYN_EXPONE_CURRENT = 4  # expCurrSynapse (PyNN): current-based, instantaneous rise, single decay
SYN_EXPTHREE = 5        # expThreeSynapse: two expTwo components sharing a rise time
SYN_BLOCKING_PLASTIC = 6  # blockingPlasticSynapse: expTwo with a voltage block and short-term plasticity


@dataclass
class SynapseType:
    """A core synapse: expOneSynapse, expTwoSynapse, alphaSynapse (tau_decay
    holds its tau), alphaCurrentSynapse (tau_decay holds its tau, gbase
    its ibase in nA, erev unused), expThreeSynapse (gbase / tau_decay the
    first component's gbase1 / tauDecay1, gbase2 / tau_decay2 the second's),
    or a PyNN synapse (`form`: expCondSynapse and alphaCondSynapse as
    SYN_EXPONE and SYN_ALPHA with gbase 1 uS, erev e_rev; expCurrSynapse as
    SYN_EXPONE_CURRENT and alphaCurrSynapse as SYN_ALPHA_CURRENT with
    1 nA; tau_decay their tau_syn)."""
    name: str
    kind: int
    gbase: float          # nS (alphaCurrentSynapse, expCurrSynapse: nA)
    erev: float           # mV
    tau_decay: float      # ms
    tau_rise: float = 0.0  # ms (expTwo and expThree)
    gbase2: float = 0.0    # nS (expThree)
    tau_decay2: float = 0.0  # ms (expThree)
    form: str = ""         # the NeuroML element a PyNN synapse was read from
    # blockingPlasticSynapse: its mechanisms' type and parameters (mM, mV,
    # ms, dimensionless), or None
    block: Optional[dict] = None
    plasticity: Optional[dict] = None


@dataclass
class Population:
    name: str
    cell_type: str        # name of a PhysicalCell or Izhikevich2007Cell
    size: int


@dataclass
class Projection:
    """connectionWD list with one synapse type.  Cells are global cell ids
    (gids: population declaration order, then index); the NeuroML writer
    splits a projection per (pre population, post population) pair."""
    name: str
    pre_pop: str
    post_pop: str
    synapse: str
    pre_cell: np.ndarray     # int index within pre_pop
    post_cell: np.ndarray    # int index within post_pop
    post_seg: np.ndarray     # int segment id on the post cell
    weight: np.ndarray       # float, dimensionless
    delay: np.ndarray        # float, ms
    conn_ids: Optional[list] = None   # per connection, (projection id, connection id) as read from NeuroML


@dataclass
class GapJunctionType:
    """A synaptic component for the ends of electrical and continuous
    connections: gapJunction and linearGradedSynapse (a current
    conductance * (vpeer - v), conductance in nS), silentSynapse (nothing),
    or gradedSynapse (conductance nS, delta mV, k per ms, vth mV, erev mV)."""
    name: str
    conductance: float
    kind: str = "gapJunction"
    delta: float = 0.0
    k: float = 0.0
    vth: float = 0.0
    erev: float = 0.0


@dataclass
class ElectricalProjection:
    """electricalConnection(Instance)(W) list of one gapJunction type: each
    connection puts an instance on both ends -- cell gid pre_cell, segment
    pre_seg, and cell gid post_cell, segment post_seg -- and each end takes
    weight * conductance * (V_other - V_own) as synaptic current, with no
    conductance term (eden/Eden.cpp:3407-3422, 9233-9251)."""
    name: str
    synapse: str
    pre_cell: np.ndarray
    pre_seg: np.ndarray
    post_cell: np.ndarray
    post_seg: np.ndarray
    weight: np.ndarray


@dataclass
class ContinuousProjection:
    """continuousConnection(Instance)(W) list: each connection puts
    `pre_component` on the pre end and `post_component` on the post end
    (GapJunctionType names), each end reading the other end's potential."""
    name: str
    pre_component: str
    post_component: str
    pre_cell: np.ndarray
    pre_seg: np.ndarray
    post_cell: np.ndarray
    post_seg: np.ndarray
    weight: np.ndarray


@dataclass
class PulseInputs:
    """One pulseGenerator per entry (delay/duration ms, amplitude nA) on
    cell gid `cell`, segment `seg`, scaled by `weight` (an inputW's; 1 when
    None)."""
    pop: str
    cell: np.ndarray
    seg: np.ndarray
    delay: np.ndarray
    duration: np.ndarray
    amplitude: np.ndarray
    weight: Optional[np.ndarray] = None
    dimensionless: bool = False   # pulseGeneratorDL (amplitude without unit, into izhikevichCell)
    list_ids: Optional[list] = None   # per input, (inputList id, input id) as read from NeuroML


@dataclass
class ClampInputs:
    """voltageClamp (`triple` False: clamps to `v_during` from `delay` for
    `duration`, no current otherwise) or voltageClampTriple (True, active:
    `v_before`, `v_during`, `v_after`) instances (ms, mV, series resistance
    `resistance` MOhm) on cell gid `cell`, segment `seg`, scaled by `weight`."""
    triple: bool
    cell: np.ndarray
    seg: np.ndarray
    delay: np.ndarray
    duration: np.ndarray
    v_before: np.ndarray
    v_during: np.ndarray
    v_after: np.ndarray
    resistance: np.ndarray
    weight: np.ndarray
    list_ids: Optional[list] = None   # per input, (inputList id, input id) as read from NeuroML


@dataclass
class PoissonInputs:
    """poissonFiringSynapse instances (`rate` Hz, each driving its own
    instance of `synapse`) on cell gid `cell`, segment `seg`.  The order of
    a spec's entries is the order the components are defined in."""
    pop: str
    synapse: str
    rate: float
    cell: np.ndarray
    seg: np.ndarray


WAVE_SINE = "sine"
WAVE_RAMP = "ramp"


@dataclass
class WaveInputs:
    """sineGenerator (shape "sine": p0 amplitude nA, p1 period ms, p2 phase)
    or rampGenerator (shape "ramp": p0 startAmplitude, p1 finishAmplitude,
    p2 baselineAmplitude, nA) instances, active from `delay` for `duration`
    (ms), on cell gid `cell`, segment `seg`, scaled by `weight`."""
    shape: str
    cell: np.ndarray
    seg: np.ndarray
    delay: np.ndarray
    duration: np.ndarray
    p0: np.ndarray
    p1: np.ndarray
    p2: np.ndarray
    weight: np.ndarray
    dimensionless: bool = False   # sine/rampGeneratorDL (amplitudes without unit, into izhikevichCell)
    list_ids: Optional[list] = None   # per input, (inputList id, input id) as read from NeuroML


@dataclass
class OutputColumn:
    pop: str
    cell: int
    seg: int
    quantity: str = "v"   # "v", or "q:<channelDensity id>/<gate id>" for a gate's state


@dataclass
class EventSelection:
    pop: str
    cell: int
    seg: int = 0


@dataclass
class TimedInputs:
    """timedSynapticInput instances: input i drives its own instance of
    `synapse` on cell gid cell[i], segment seg[i], firing at times[i] (ms),
    scaled by weight[i]."""
    synapse: str
    cell: np.ndarray
    seg: np.ndarray
    times: list
    weight: np.ndarray


@dataclass
class NetworkSpec:
    name: str
    dt: float               # ms
    length: float           # ms
    seed: int
    channels: List[Channel] = field(default_factory=list)
    cells: list = field(default_factory=list)           # PhysicalCell | Izhikevich2007Cell
    synapses: List[SynapseType] = field(default_factory=list)
    populations: List[Population] = field(default_factory=list)
    projections: List[Projection] = field(default_factory=list)
    gap_types: List[GapJunctionType] = field(default_factory=list)
    electrical: List[ElectricalProjection] = field(default_factory=list)
    continuous: List[ContinuousProjection] = field(default_factory=list)
    pulses: List[PulseInputs] = field(default_factory=list)
    poissons: List[PoissonInputs] = field(default_factory=list)
    timed: List[TimedInputs] = field(default_factory=list)
    waves: List[WaveInputs] = field(default_factory=list)
    clamps: List[ClampInputs] = field(default_factory=list)
    temperature: float = 6.3  # degC: the network's, or the reference's default when it has none
    custom_setup: list = field(default_factory=list)   # EdenCustomSetup statements (custom_setup.SetCell)
    trace_columns: List[OutputColumn] = field(default_factory=list)
    trace_file: str = "trajectory.txt"
    event_selections: List[EventSelection] = field(default_factory=list)
    event_file: str = "spikes.txt"
    event_format: str = "TIME_ID"
    cable_solver: str = "auto"   # the reference's cable_solver setting: auto (= bwd_euler), bwd_euler, fwd_euler

    # -- lookups ---------------------------------------------------------
    def _index(self, attr: str, items) -> dict:
        # name -> item, rebuilt when the list changed length
        cache = self.__dict__.setdefault("_lookup", {})
        hit = cache.get(attr)
        if hit is None or hit[0] != len(items):
            hit = (len(items), {x.name: x for x in reversed(items)})
            cache[attr] = hit
        return hit[1]

    def cell_type(self, name: str):
        try:
            return self._index("cells", self.cells)[name]
        except KeyError:
            raise KeyError(name) from None

    def synapse(self, name: str) -> SynapseType:
        try:
            return self._index("synapses", self.synapses)[name]
        except KeyError:
            raise KeyError(name) from None

    def population(self, name: str) -> Population:
        try:
            return self._index("populations", self.populations)[name]
        except KeyError:
            raise KeyError(name) from None

    def pop_offsets(self) -> dict:
        """Global cell id (gid) of each population's first cell, in
        declaration order (the reference's work-item order)."""
        off, out = 0, {}
        for p in self.populations:
            out[p.name] = off
            off += p.size
        return out

    @property
    def n_cells(self) -> int:
        return sum(p.size for p in self.populations)

    def n_compartments(self) -> int:
        total = 0
        for p in self.populations:
            ct = self.cell_type(p.cell_type)
            total += p.size * (ct.n_seg if isinstance(ct, PhysicalCell) else
                               0 if isinstance(ct, SPIKE_SOURCE_TYPES) else 1)
        return total

    def n_synapses(self) -> int:
        return int(sum(len(pr.pre_cell) for pr in self.projections))

    def n_poisson(self) -> int:
        return int(sum(len(pi.cell) for pi in self.poissons))

    def n_steps(self) -> int:
        """Non-initialisation steps: t = 0, dt, ... while t <= length
        (eden/Eden.cpp:11488)."""
        dt_us = np.float32(self.dt * 1000.0)
        t_final = self.length * 1000.0
        n, t = 0, 0.0
        # times are exact multiples of dt in the configurations used here
        n = int(np.floor(t_final / float(dt_us) + 1e-9)) + 1
        return n
