"""LEMS/NeuroML files <-> NetworkSpec.

`write_lems(spec, dirname)` writes `<name>.nml` (the NeuroML model) and
`LEMS_<name>.xml` (the simulation with its OutputFile/EventOutputFile) in the
form the reference simulator reads (`eden nml LEMS_<name>.xml`).

`read_lems(path)` reads such a file back into a NetworkSpec.  It covers the
subset of NeuroML2/LEMS this path simulates (see network.py) and rejects
anything else with a ValueError naming the element, so an unsupported model
fails loudly instead of being simulated wrongly.
"""
from __future__ import annotations

import os
import re
import xml.etree.ElementTree as ET
from collections import defaultdict

import numpy as np

from .network import (Channel, ChannelDensity, EventSelection, Gate,
                      Izhikevich2007Cell, NetworkSpec, OutputColumn,
                      PhysicalCell, PoissonInputs, Population, Projection,
                      PulseInputs, Rate, SynapseType, RATE_TYPE_NAMES,
                      SYN_EXPONE, SYN_EXPTWO)


def _f(x: float) -> str:
    return repr(float(x))


def _gid_maps(spec: NetworkSpec):
    pops, local = [], []
    for p in spec.populations:
        pops.extend([p.name] * p.size)
        local.extend(range(p.size))
    return np.array(pops, dtype=object), np.array(local, dtype=np.int64)


def write_lems(spec: NetworkSpec, dirname: str) -> str:
    """Write the model and simulation files; returns the LEMS file path."""
    os.makedirs(dirname, exist_ok=True)
    nml_name = f"{spec.name}.nml"
    lems_path = os.path.join(dirname, f"LEMS_{spec.name}.xml")
    out = []
    w = out.append
    w('<?xml version="1.0" encoding="UTF-8"?>\n')
    w(f'<neuroml xmlns="http://www.neuroml.org/schema/neuroml2" id="{spec.name}">\n')
    for ch in spec.channels:
        sp = f' species="{ch.species}"' if ch.species else ""
        if not ch.gates:
            w(f'<ionChannelHH id="{ch.name}" conductance="10pS"{sp}/>\n')
            continue
        w(f'<ionChannelHH id="{ch.name}" conductance="10pS"{sp}>\n')
        for g in ch.gates:
            w(f' <gateHHrates id="{g.name}" instances="{g.instances}">\n')
            for tag, r in (("forwardRate", g.forward), ("reverseRate", g.reverse)):
                w(f'  <{tag} type="{RATE_TYPE_NAMES[r.kind]}" rate="{_f(r.rate)}per_ms" '
                  f'midpoint="{_f(r.midpoint)}mV" scale="{_f(r.scale)}mV"/>\n')
            w(' </gateHHrates>\n')
        w('</ionChannelHH>\n')
    for s in spec.synapses:
        if s.kind == SYN_EXPONE:
            w(f'<expOneSynapse id="{s.name}" gbase="{_f(s.gbase)}nS" erev="{_f(s.erev)}mV" '
              f'tauDecay="{_f(s.tau_decay)}ms"/>\n')
        else:
            w(f'<expTwoSynapse id="{s.name}" gbase="{_f(s.gbase)}nS" erev="{_f(s.erev)}mV" '
              f'tauRise="{_f(s.tau_rise)}ms" tauDecay="{_f(s.tau_decay)}ms"/>\n')
    used_types = {p.cell_type for p in spec.populations}
    for c in spec.cells:
        if c.name not in used_types:
            continue
        if isinstance(c, Izhikevich2007Cell):
            w(f'<izhikevich2007Cell id="{c.name}" v0="{_f(c.v0)}mV" C="{_f(c.C)}pF" '
              f'k="{_f(c.k)}nS_per_mV" vr="{_f(c.vr)}mV" vt="{_f(c.vt)}mV" vpeak="{_f(c.vpeak)}mV" '
              f'a="{_f(c.a)}per_ms" b="{_f(c.b)}nS" c="{_f(c.c)}mV" d="{_f(c.d)}pA"/>\n')
        else:
            _write_cell(w, spec, c)
    # inputs: one pulseGenerator per distinct (delay, duration, amplitude)
    pulse_ids = {}
    for pi in spec.pulses:
        for d, du, a in zip(pi.delay, pi.duration, pi.amplitude):
            key = (float(d), float(du), float(a))
            if key not in pulse_ids:
                pid = f"pg{len(pulse_ids)}"
                pulse_ids[key] = pid
                w(f'<pulseGenerator id="{pid}" delay="{_f(d)}ms" duration="{_f(du)}ms" amplitude="{_f(a)}nA"/>\n')
    pois_ids = {}
    for k, po in enumerate(spec.poissons):
        pid = f"poisson{k}"
        pois_ids[k] = pid
        w(f'<poissonFiringSynapse id="{pid}" averageRate="{_f(po.rate)} Hz" synapse="{po.synapse}" '
          f'spikeTarget="./{po.synapse}"/>\n')

    w('<network id="net">\n')
    for p in spec.populations:
        w(f' <population id="{p.name}" component="{p.cell_type}" size="{p.size}"/>\n')
    pop_of, local_of = _gid_maps(spec)
    for pr in spec.projections:
        groups = defaultdict(list)
        for i in range(len(pr.pre_cell)):
            groups[(pop_of[pr.pre_cell[i]], pop_of[pr.post_cell[i]])].append(i)
        for gi, ((pa, pb), idx) in enumerate(groups.items()):
            w(f' <projection id="{pr.name}_{gi}" presynapticPopulation="{pa}" '
              f'postsynapticPopulation="{pb}" synapse="{pr.synapse}">\n')
            for n, i in enumerate(idx):
                w(f'  <connectionWD id="{n}" preCellId="../{pa}[{local_of[pr.pre_cell[i]]}]" '
                  f'postCellId="../{pb}[{local_of[pr.post_cell[i]]}]" postSegmentId="{pr.post_seg[i]}" '
                  f'weight="{_f(pr.weight[i])}" delay="{_f(pr.delay[i])}ms"/>\n')
            w(' </projection>\n')
    n_list = 0
    for pi in spec.pulses:
        by_comp = defaultdict(list)
        for i in range(len(pi.cell)):
            key = (float(pi.delay[i]), float(pi.duration[i]), float(pi.amplitude[i]))
            by_comp[(pulse_ids[key], pop_of[pi.cell[i]])].append(i)
        for (pid, pop), idx in by_comp.items():
            w(f' <inputList id="il{n_list}" component="{pid}" population="{pop}">\n')
            n_list += 1
            for n, i in enumerate(idx):
                w(f'  <input id="{n}" target="../{pop}[{local_of[pi.cell[i]]}]" segmentId="{pi.seg[i]}" '
                  f'fractionAlong="0.5" destination="synapses"/>\n')
            w(' </inputList>\n')
    for k, po in enumerate(spec.poissons):
        by_pop = defaultdict(list)
        for i in range(len(po.cell)):
            by_pop[pop_of[po.cell[i]]].append(i)
        for pop, idx in by_pop.items():
            w(f' <inputList id="il{n_list}" component="{pois_ids[k]}" population="{pop}">\n')
            n_list += 1
            for n, i in enumerate(idx):
                w(f'  <input id="{n}" target="../{pop}[{local_of[po.cell[i]]}]" segmentId="{po.seg[i]}" '
                  f'fractionAlong="0.5" destination="synapses"/>\n')
            w(' </inputList>\n')
    w('</network>\n</neuroml>\n')
    with open(os.path.join(dirname, nml_name), "w") as f:
        f.write("".join(out))

    # the LEMS simulation file
    lw = []
    lw.append('<Lems>\n<Target component="sim"/>\n')
    lw.append('<Include file="Cells.xml"/>\n<Include file="Networks.xml"/>\n<Include file="Simulation.xml"/>\n')
    lw.append(f'<Include file="{nml_name}"/>\n')
    lw.append(f'<Simulation id="sim" length="{_f(spec.length)}ms" step="{_f(spec.dt)}ms" target="net" seed="{spec.seed}">\n')
    if spec.trace_columns:
        lw.append(f' <OutputFile id="traj" fileName="{spec.trace_file}">\n')
        for i, col in enumerate(spec.trace_columns):
            lw.append(f'  <OutputColumn id="c{i}" quantity="{_quantity_path(spec, col)}"/>\n')
        lw.append(' </OutputFile>\n')
    if spec.event_selections:
        lw.append(f' <EventOutputFile id="spk" fileName="{spec.event_file}" format="{spec.event_format}">\n')
        for i, ev in enumerate(spec.event_selections):
            lw.append(f'  <EventSelection id="{i}" select="{_select_path(spec, ev)}" eventPort="spike"/>\n')
        lw.append(' </EventOutputFile>\n')
    lw.append('</Simulation>\n</Lems>\n')
    with open(lems_path, "w") as f:
        f.write("".join(lw))
    return lems_path


def _quantity_path(spec, col: OutputColumn) -> str:
    ct = spec.cell_type(spec.population(col.pop).cell_type)
    if isinstance(ct, PhysicalCell):
        return f"{col.pop}/{col.cell}/{ct.name}/{col.seg}/v"
    return f"{col.pop}/{col.cell}/{ct.name}/v"


def _select_path(spec, ev: EventSelection) -> str:
    ct = spec.cell_type(spec.population(ev.pop).cell_type)
    if isinstance(ct, PhysicalCell):
        return f"{ev.pop}/{ev.cell}/{ct.name}/{ev.seg}"
    return f"{ev.pop}/{ev.cell}/{ct.name}"


def _write_cell(w, spec: NetworkSpec, c: PhysicalCell) -> None:
    w(f'<cell id="{c.name}">\n <morphology id="{c.name}_morph">\n')
    # cylinders laid out along +x from the parent's distal point
    dist_x = np.zeros(c.n_seg)
    for i in range(c.n_seg):
        p = int(c.seg_parent[i])
        x0 = 0.0 if p < 0 else dist_x[p]
        dist_x[i] = x0 + float(c.seg_len[i])
        if p < 0:
            w(f'  <segment id="{i}" name="seg{i}">\n'
              f'   <proximal x="{_f(x0)}" y="0" z="0" diameter="{_f(c.seg_diam[i])}"/>\n'
              f'   <distal x="{_f(dist_x[i])}" y="0" z="0" diameter="{_f(c.seg_diam[i])}"/>\n  </segment>\n')
        else:
            w(f'  <segment id="{i}" name="seg{i}">\n   <parent segment="{p}"/>\n'
              f'   <proximal x="{_f(x0)}" y="0" z="0" diameter="{_f(c.seg_diam[i])}"/>\n'
              f'   <distal x="{_f(dist_x[i])}" y="0" z="0" diameter="{_f(c.seg_diam[i])}"/>\n  </segment>\n')
    groups = dict(c.seg_groups)
    group_of_mask = {}
    for gname, mask in groups.items():
        if mask.any():
            w(f'  <segmentGroup id="{gname}">\n')
            for i in np.nonzero(mask)[0]:
                w(f'   <member segment="{int(i)}"/>\n')
            w('  </segmentGroup>\n')
        group_of_mask[np.asarray(mask, bool).tobytes()] = gname
    w(' </morphology>\n <biophysicalProperties id="bio">\n  <membraneProperties>\n')
    for k, d in enumerate(c.densities):
        if not d.seg_mask.any():
            continue
        ch = spec.channels[d.channel]
        ion = ch.species or "non_specific"
        if d.seg_mask.all():
            sg = ""
        else:
            gname = group_of_mask.get(np.asarray(d.seg_mask, bool).tobytes())
            if gname is None:
                raise ValueError(f"cell {c.name}: channel density {k} has no matching segment group")
            sg = f' segmentGroup="{gname}"'
        w(f'   <channelDensity id="cd{k}" ionChannel="{ch.name}" condDensity="{_f(d.cond)} mS_per_cm2" '
          f'erev="{_f(d.erev)}mV" ion="{ion}"{sg}/>\n')
    w(f'   <spikeThresh value="{_f(c.spike_thresh)}mV"/>\n')
    w(f'   <specificCapacitance value="{_f(c.cm)} uF_per_cm2"/>\n')
    w(f'   <initMembPotential value="{_f(c.v0)}mV"/>\n')
    w('  </membraneProperties>\n  <intracellularProperties>\n')
    w(f'   <resistivity value="{_f(c.ra)} ohm_cm"/>\n')
    w('  </intracellularProperties>\n </biophysicalProperties>\n</cell>\n')
