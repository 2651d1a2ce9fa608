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
                      PulseInputs, Rate, SpikeArrayCell, SpikeGeneratorCell, SpikeGeneratorPoissonCell,
                      SpikeGeneratorRandomCell, SynapseType,
                      EventSetReaderCell,
                      RATE_TYPE_NAMES, SYN_EXPONE, SYN_EXPTWO, WAVE_SINE, WAVE_RAMP, AdExCell, IafCell,
                      ClampInputs, FitzHughNagumoCell, IzhikevichCell, TimedInputs, WaveInputs,
                      ElectricalProjection, GapJunctionType, SYN_ALPHA, SYN_ALPHA_CURRENT,
                      SYN_EXPONE_CURRENT, SYN_EXPTHREE, ContinuousProjection, SYN_BLOCKING_PLASTIC)


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
            tag = _GATE_TAGS[g.kind]
            w(f' <{tag} id="{g.name}" instances="{g.instances}">\n')
            if g.q10 is not None:
                if g.q10[0] == "fixed":
                    w(f'  <q10Settings type="q10Fixed" fixedQ10="{_f(g.q10[1])}"/>\n')
                else:
                    w(f'  <q10Settings type="q10ExpTemp" q10Factor="{_f(g.q10[1])}" '
                      f'experimentalTemp="{_f(g.q10[2])} degC"/>\n')
            if g.forward is not None:
                for rtag, r in (("forwardRate", g.forward), ("reverseRate", g.reverse)):
                    w(f'  <{rtag} type="{RATE_TYPE_NAMES[r.kind]}" rate="{_f(r.rate)}per_ms" '
                      f'midpoint="{_f(r.midpoint)}mV" scale="{_f(r.scale)}mV"/>\n')
            if g.tau is not None:
                w(f'  <timeCourse type="fixedTimeCourse" tau="{_f(g.tau)}ms"/>\n')
            if g.inf is not None:
                w(f'  <steadyState type="{_VARIABLE_TYPE_NAMES[g.inf.kind]}" rate="{_f(g.inf.rate)}" '
                  f'midpoint="{_f(g.inf.midpoint)}mV" scale="{_f(g.inf.scale)}mV"/>\n')
            w(f' </{tag}>\n')
        w('</ionChannelHH>\n')
    for s in spec.synapses:
        if s.form:
            cond = _PYNN_SYNAPSES[s.form][1]
            w(f'<{s.form} id="{s.name}" tau_syn="{_f(s.tau_decay)}"' + (f' e_rev="{_f(s.erev)}"' if cond else '')
              + '/>\n')
        elif s.kind == SYN_BLOCKING_PLASTIC:
            w(f'<blockingPlasticSynapse id="{s.name}" gbase="{_f(s.gbase)}nS" erev="{_f(s.erev)}mV" '
              f'tauRise="{_f(s.tau_rise)}ms" tauDecay="{_f(s.tau_decay)}ms">\n')
            if s.block:
                b = s.block
                w(f' <blockMechanism type="voltageConcDepBlockMechanism" species="{b.get("species") or "mg"}" '
                  f'blockConcentration="{_f(b["blockConcentration"])}mM" scalingConc="{_f(b["scalingConc"])}mM" '
                  f'scalingVolt="{_f(b["scalingVolt"])}mV"/>\n')
            if s.plasticity:
                pl = s.plasticity
                w(f' <plasticityMechanism type="{pl["type"]}" initReleaseProb="{_f(pl["initReleaseProb"])}" '
                  f'tauRec="{_f(pl["tauRec"])}ms"' + (f' tauFac="{_f(pl["tauFac"])}ms"' if "tauFac" in pl else "")
                  + '/>\n')
            w('</blockingPlasticSynapse>\n')
        elif s.kind == SYN_EXPTHREE:
            w(f'<expThreeSynapse id="{s.name}" gbase1="{_f(s.gbase)}nS" gbase2="{_f(s.gbase2)}nS" '
              f'erev="{_f(s.erev)}mV" tauRise="{_f(s.tau_rise)}ms" tauDecay1="{_f(s.tau_decay)}ms" '
              f'tauDecay2="{_f(s.tau_decay2)}ms"/>\n')
        elif s.kind == SYN_EXPONE_CURRENT:
            raise ValueError(f"synapse {s.name}: a current-based single-exponential synapse is written as "
                             f"expCurrSynapse (form), whose jump is 1 nA")
        elif s.kind == SYN_EXPONE:
            w(f'<expOneSynapse id="{s.name}" gbase="{_f(s.gbase)}nS" erev="{_f(s.erev)}mV" '
              f'tauDecay="{_f(s.tau_decay)}ms"/>\n')
        elif s.kind == SYN_ALPHA:
            w(f'<alphaSynapse id="{s.name}" gbase="{_f(s.gbase)}nS" erev="{_f(s.erev)}mV" '
              f'tau="{_f(s.tau_decay)}ms"/>\n')
        elif s.kind == SYN_ALPHA_CURRENT:
            w(f'<alphaCurrentSynapse id="{s.name}" ibase="{_f(s.gbase)}nA" tau="{_f(s.tau_decay)}ms"/>\n')
        else:
            w(f'<expTwoSynapse id="{s.name}" gbase="{_f(s.gbase)}nS" erev="{_f(s.erev)}mV" '
              f'tauRise="{_f(s.tau_rise)}ms" tauDecay="{_f(s.tau_decay)}ms"/>\n')
    for gt in spec.gap_types:
        if gt.kind == "silentSynapse":
            w(f'<silentSynapse id="{gt.name}"/>\n')
        elif gt.kind == "gradedSynapse":
            w(f'<gradedSynapse id="{gt.name}" conductance="{_f(gt.conductance)}nS" delta="{_f(gt.delta)}mV" '
              f'k="{_f(gt.k)}per_ms" Vth="{_f(gt.vth)}mV" erev="{_f(gt.erev)}mV"/>\n')
        else:
            w(f'<{gt.kind} id="{gt.name}" conductance="{_f(gt.conductance)}nS"/>\n')
    used_types = {p.cell_type for p in spec.populations}
    for c in spec.cells:
        if c.name not in used_types:
            continue
        if isinstance(c, EventSetReaderCell):
            continue                      # written in the network
        if isinstance(c, SpikeArrayCell):
            w(f'<spikeArray id="{c.name}">')
            for i, t in enumerate(c.times):
                w(f'<spike id="{i}" time="{_f(t)}ms"/>')
            w('</spikeArray>\n')
        elif isinstance(c, SpikeGeneratorCell):
            w(f'<spikeGenerator id="{c.name}" period="{_f(c.period)}ms"/>\n')
        elif isinstance(c, SpikeGeneratorRandomCell):
            w(f'<spikeGeneratorRandom id="{c.name}" minISI="{_f(c.min_isi)}ms" maxISI="{_f(c.max_isi)}ms"/>\n')
        elif isinstance(c, SpikeGeneratorPoissonCell):
            if c.min_isi is None:
                w(f'<spikeGeneratorPoisson id="{c.name}" averageRate="{_f(c.rate)} Hz"/>\n')
            else:
                w(f'<spikeGeneratorRefPoisson id="{c.name}" averageRate="{_f(c.rate)} Hz" '
                  f'minimumISI="{_f(c.min_isi)}ms"/>\n')
        elif isinstance(c, IafCell):
            extra = ""
            if c.kind in ("iafTauCell", "iafTauRefCell"):
                extra += f' tau="{_f(c.tau)}ms"'
            else:
                extra += f' C="{_f(c.C)}pF" leakConductance="{_f(c.leak_conductance)}nS"'
            if c.kind.endswith("RefCell"):
                extra += f' refract="{_f(c.refract)}ms"'
            w(f'<{c.kind} id="{c.name}" leakReversal="{_f(c.leak_reversal)}mV" thresh="{_f(c.thresh)}mV" '
              f'reset="{_f(c.reset)}mV"{extra}/>\n')
        elif isinstance(c, AdExCell):
            w(f'<adExIaFCell id="{c.name}" C="{_f(c.C)}pF" gL="{_f(c.gL)}nS" EL="{_f(c.EL)}mV" VT="{_f(c.VT)}mV" '
              f'thresh="{_f(c.thresh)}mV" reset="{_f(c.reset)}mV" delT="{_f(c.delT)}mV" tauw="{_f(c.tauw)}ms" '
              f'refract="{_f(c.refract)}ms" a="{_f(c.a)}nS" b="{_f(c.b)}nA"/>\n')
        elif isinstance(c, FitzHughNagumoCell):
            w(f'<fitzHughNagumoCell id="{c.name}" I="{_f(c.I)}"/>\n')
        elif isinstance(c, IzhikevichCell):
            w(f'<izhikevichCell id="{c.name}" v0="{_f(c.v0)}mV" thresh="{_f(c.thresh)}mV" a="{_f(c.a)}" '
              f'b="{_f(c.b)}" c="{_f(c.c)}" d="{_f(c.d)}"/>\n')
        elif isinstance(c, Izhikevich2007Cell):
            w(f'<izhikevich2007Cell id="{c.name}" v0="{_f(c.v0)}mV" C="{_f(c.C)}pF" '
              f'k="{_f(c.k)}nS_per_mV" vr="{_f(c.vr)}mV" vt="{_f(c.vt)}mV" vpeak="{_f(c.vpeak)}mV" '
              f'a="{_f(c.a)}per_ms" b="{_f(c.b)}nS" c="{_f(c.c)}mV" d="{_f(c.d)}pA"/>\n')
        else:
            _write_cell(w, spec, c)
    # inputs: one pulseGenerator per distinct (delay, duration, amplitude)
    pulse_ids = {}
    for pi in spec.pulses:
        for d, du, a in zip(pi.delay, pi.duration, pi.amplitude):
            key = (float(d), float(du), float(a), pi.dimensionless)
            if key not in pulse_ids:
                pid = f"pg{len(pulse_ids)}"
                pulse_ids[key] = pid
                if pi.dimensionless:
                    w(f'<pulseGeneratorDL id="{pid}" delay="{_f(d)}ms" duration="{_f(du)}ms" amplitude="{_f(a)}"/>\n')
                else:
                    w(f'<pulseGenerator id="{pid}" delay="{_f(d)}ms" duration="{_f(du)}ms" '
                      f'amplitude="{_f(a)}nA"/>\n')
    pois_ids = {}
    for k, po in enumerate(spec.poissons):
        pid = f"poisson{k}"
        pois_ids[k] = pid
        w(f'<poissonFiringSynapse id="{pid}" averageRate="{_f(po.rate)} Hz" synapse="{po.synapse}" '
          f'spikeTarget="./{po.synapse}"/>\n')

    timed_ids = []
    for k, ti in enumerate(spec.timed):
        for i, times in enumerate(ti.times):
            tid = f"timed{k}_{i}"
            timed_ids.append((tid, k, i))
            w(f'<timedSynapticInput id="{tid}" synapse="{ti.synapse}" spikeTarget="./{ti.synapse}">')
            for j, t in enumerate(times):
                w(f'<spike id="{j}" time="{_f(t)}ms"/>')
            w('</timedSynapticInput>\n')
    # sine / ramp generators: one component per distinct parameter set
    wave_ids = {}
    for wv in spec.waves:
        for i in range(len(wv.cell)):
            key = _wave_key(wv, i)
            if key in wave_ids:
                continue
            wid = f"wave{len(wave_ids)}"
            wave_ids[key] = wid
            _, d, du, a, b, c = key
            dl, na = ("DL", "") if wv.dimensionless else ("", "nA")
            if wv.shape == WAVE_SINE:
                w(f'<sineGenerator{dl} id="{wid}" delay="{_f(d)}ms" duration="{_f(du)}ms" amplitude="{_f(a)}{na}" '
                  f'period="{_f(b)}ms" phase="{_f(c)}"/>\n')
            else:
                w(f'<rampGenerator{dl} id="{wid}" delay="{_f(d)}ms" duration="{_f(du)}ms" '
                  f'startAmplitude="{_f(a)}{na}" finishAmplitude="{_f(b)}{na}" baselineAmplitude="{_f(c)}{na}"/>\n')
    clamp_ids = {}
    for cl in spec.clamps:
        for i in range(len(cl.cell)):
            key = _clamp_key(cl, i)
            if key in clamp_ids:
                continue
            cid = f"clamp{len(clamp_ids)}"
            clamp_ids[key] = cid
            _, d, du, vb, vd, va, r = key
            if cl.triple:
                w(f'<voltageClampTriple id="{cid}" delay="{_f(d)}ms" duration="{_f(du)}ms" active="1" '
                  f'conditioningVoltage="{_f(vb)}mV" testingVoltage="{_f(vd)}mV" returnVoltage="{_f(va)}mV" '
                  f'simpleSeriesResistance="{_f(r)}Mohm"/>\n')
            else:
                w(f'<voltageClamp id="{cid}" delay="{_f(d)}ms" duration="{_f(du)}ms" targetVoltage="{_f(vd)}mV" '
                  f'simpleSeriesResistance="{_f(r)}Mohm"/>\n')
    if spec.temperature != 6.3 or any(g.q10 is not None and g.q10[0] == "exp" for ch in spec.channels
                                      for g in ch.gates):
        w(f'<network id="net" type="networkWithTemperature" temperature="{_f(spec.temperature)} degC">\n')
    else:
        w('<network id="net">\n')
    readers = {}
    for p in spec.populations:
        ct = spec.cell_type(p.cell_type)
        if isinstance(ct, EventSetReaderCell):
            readers[p.name] = ct
            continue
        w(f' <population id="{p.name}" component="{p.cell_type}" size="{p.size}"/>\n')
    for name, ct in readers.items():
        w(f' <EdenEventSetReader id="{name}" href="./{ct.href}" format="ascii_v0" instances="{ct.instances}">\n')
        for port in ct.ports:
            w(f'  <Port id="{port}"/>\n')
        w(' </EdenEventSetReader>\n')
        with open(os.path.join(dirname, ct.href), "w") as f:
            for ts, pairs in ct.frames:
                f.write(repr(float(ts)) + "".join(f" {i}!{q}" for i, q in pairs) + "\n")
    pop_of, local_of = _gid_maps(spec)
    for pr in spec.projections:
        # consecutive runs of one (pre, post) population pair -- and, where the
        # connections carry the (projection id, connection id) they were read
        # with, of one such projection, so `set synapse` statements still
        # name them -- so the file's connection order, the reference's
        # instantiation order, is the projection's own
        ids = pr.conn_ids
        groups = []
        for i in range(len(pr.pre_cell)):
            key = (pop_of[pr.pre_cell[i]], pop_of[pr.post_cell[i]], ids[i][0] if ids else None)
            if not groups or groups[-1][0] != key:
                groups.append((key, []))
            groups[-1][1].append(i)
        for gi, ((pa, pb, pid), idx) in enumerate(groups):
            w(f' <projection id="{pid if ids else f"{pr.name}_{gi}"}" presynapticPopulation="{pa}" '
              f'postsynapticPopulation="{pb}" synapse="{pr.synapse}">\n')
            for n0, i in enumerate(idx):
                n = ids[i][1] if ids else n0
                if pa in readers:
                    inst, port = divmod(local_of[pr.pre_cell[i]], len(readers[pa].ports))
                    w(f'  <connectionWD id="{n}" preCellId="{inst}" preSegmentId="{readers[pa].ports[port]}" '
                      f'postCellId="../{pb}[{local_of[pr.post_cell[i]]}]" postSegmentId="{pr.post_seg[i]}" '
                      f'weight="{_f(pr.weight[i])}" delay="{_f(pr.delay[i])}ms"/>\n')
                    continue
                w(f'  <connectionWD id="{n}" preCellId="../{pa}[{local_of[pr.pre_cell[i]]}]" '
                  f'postCellId="../{pb}[{local_of[pr.post_cell[i]]}]" postSegmentId="{pr.post_seg[i]}" '
                  f'weight="{_f(pr.weight[i])}" delay="{_f(pr.delay[i])}ms"/>\n')
            w(' </projection>\n')
    for ep in spec.electrical:
        # one electricalProjection per (pre population, post population) run
        groups = []
        for i in range(len(ep.pre_cell)):
            key = (pop_of[ep.pre_cell[i]], pop_of[ep.post_cell[i]])
            if not groups or groups[-1][0] != key:
                groups.append((key, []))
            groups[-1][1].append(i)
        for gi, ((pa, pb), idx) in enumerate(groups):
            w(f' <electricalProjection id="{ep.name}_{gi}" presynapticPopulation="{pa}" '
              f'postsynapticPopulation="{pb}">\n')
            for n, i in enumerate(idx):
                w(f'  <electricalConnectionInstanceW id="{n}" preCell="../{pa}/{local_of[ep.pre_cell[i]]}/'
                  f'{spec.population(pa).cell_type}" preSegment="{ep.pre_seg[i]}" '
                  f'postCell="../{pb}/{local_of[ep.post_cell[i]]}/{spec.population(pb).cell_type}" '
                  f'postSegment="{ep.post_seg[i]}" synapse="{ep.synapse}" weight="{_f(ep.weight[i])}"/>\n')
            w(' </electricalProjection>\n')
    for cp in spec.continuous:
        # one continuousProjection per (pre population, post population) run
        groups = []
        for i in range(len(cp.pre_cell)):
            key = (pop_of[cp.pre_cell[i]], pop_of[cp.post_cell[i]])
            if not groups or groups[-1][0] != key:
                groups.append((key, []))
            groups[-1][1].append(i)
        for gi, ((pa, pb), idx) in enumerate(groups):
            w(f' <continuousProjection id="{cp.name}_{gi}" presynapticPopulation="{pa}" '
              f'postsynapticPopulation="{pb}">\n')
            for n, i in enumerate(idx):
                w(f'  <continuousConnectionInstanceW id="{n}" preCell="../{pa}/{local_of[cp.pre_cell[i]]}/'
                  f'{spec.population(pa).cell_type}" preSegment="{cp.pre_seg[i]}" '
                  f'postCell="../{pb}/{local_of[cp.post_cell[i]]}/{spec.population(pb).cell_type}" '
                  f'postSegment="{cp.post_seg[i]}" preComponent="{cp.pre_component}" '
                  f'postComponent="{cp.post_component}" weight="{_f(cp.weight[i])}"/>\n')
            w(' </continuousProjection>\n')
    n_list = 0

    def input_lists(obj, comp_of, weighted):
        # one inputList per component and population, or the lists (and
        # input ids) the items were read from
        nonlocal n_list
        by_comp = defaultdict(list)
        for i in range(len(obj.cell)):
            lname = obj.list_ids[i][0] if obj.list_ids else None
            by_comp[(comp_of(i), pop_of[obj.cell[i]], lname)].append(i)
        for (cid, pop, lname), idx in by_comp.items():
            w(f' <inputList id="{lname or f"il{n_list}"}" component="{cid}" population="{pop}">\n')
            n_list += 1
            for n, i in enumerate(idx):
                iid = obj.list_ids[i][1] if obj.list_ids else n
                tgt = f'target="../{pop}[{local_of[obj.cell[i]]}]" segmentId="{obj.seg[i]}" fractionAlong="0.5"'
                if weighted:
                    w(f'  <inputW id="{iid}" {tgt} destination="synapses" weight="{_f(obj.weight[i])}"/>\n')
                else:
                    w(f'  <input id="{iid}" {tgt} destination="synapses"/>\n')
            w(' </inputList>\n')

    for pi in spec.pulses:
        input_lists(pi, lambda i, pi=pi: pulse_ids[(float(pi.delay[i]), float(pi.duration[i]),
                                                     float(pi.amplitude[i]), pi.dimensionless)],
                    pi.weight is not None)
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
    for cl in spec.clamps:
        input_lists(cl, lambda i, cl=cl: clamp_ids[_clamp_key(cl, i)], True)
    for wv in spec.waves:
        input_lists(wv, lambda i, wv=wv: wave_ids[_wave_key(wv, i)], True)
    for tid, k, i in timed_ids:
        ti = spec.timed[k]
        pop = pop_of[ti.cell[i]]
        w(f' <inputList id="il{n_list}" component="{tid}" population="{pop}">\n')
        n_list += 1
        w(f'  <inputW id="0" target="../{pop}[{local_of[ti.cell[i]]}]" segmentId="{ti.seg[i]}" '
          f'fractionAlong="0.5" destination="synapses" weight="{_f(ti.weight[i])}"/>\n')
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
    if spec.custom_setup:
        from .custom_setup import write as write_setup
        write_setup(spec, os.path.join(dirname, f"{spec.name}_setup.txt"))
        lw.append(f' <EdenCustomSetup filename="./{spec.name}_setup.txt"/>\n')
    lw.append('</Simulation>\n</Lems>\n')
    with open(lems_path, "w") as f:
        f.write("".join(lw))
    return lems_path


def _quantity_path(spec, col: OutputColumn) -> str:
    ct = spec.cell_type(spec.population(col.pop).cell_type)
    if isinstance(ct, PhysicalCell) and col.quantity.startswith("q:"):
        dname, gate = col.quantity[2:].split("/")
        k = next(k for k, d in enumerate(ct.densities) if (d.name or f"cd{k}") == dname)
        chan = spec.channels[ct.densities[k].channel].name
        return f"{col.pop}/{col.cell}/{ct.name}/{col.seg}/bio/membraneProperties/{dname}/{chan}/{gate}/q"
    if isinstance(ct, PhysicalCell):
        return f"{col.pop}/{col.cell}/{ct.name}/{col.seg}/v"
    # a fitzHughNagumoCell's membrane variable is the dimensionless V
    return f"{col.pop}/{col.cell}/{ct.name}/{'V' if isinstance(ct, FitzHughNagumoCell) else 'v'}"


def _select_path(spec, ev: EventSelection) -> str:
    ct = spec.cell_type(spec.population(ev.pop).cell_type)
    if isinstance(ct, PhysicalCell):
        return f"{ev.pop}/{ev.cell}/{ct.name}/{ev.seg}"
    return f"{ev.pop}/{ev.cell}/{ct.name}"


def _write_cell(w, spec: NetworkSpec, c: PhysicalCell) -> None:
    w(f'<cell id="{c.name}">\n <morphology id="{c.name}_morph">\n')
    # segments laid out along +x from the parent's distal point
    dist_x = np.zeros(c.n_seg)
    dprox = c.seg_diam if c.seg_dprox is None else c.seg_dprox
    for i in range(c.n_seg):
        p = int(c.seg_parent[i])
        x0 = 0.0 if p < 0 else dist_x[p]
        dist_x[i] = x0 + float(c.seg_len[i])
        if p < 0:
            w(f'  <segment id="{i}" name="seg{i}">\n'
              f'   <proximal x="{_f(x0)}" y="0" z="0" diameter="{_f(dprox[i])}"/>\n'
              f'   <distal x="{_f(dist_x[i])}" y="0" z="0" diameter="{_f(c.seg_diam[i])}"/>\n  </segment>\n')
        else:
            w(f'  <segment id="{i}" name="seg{i}">\n   <parent segment="{p}"/>\n'
              f'   <proximal x="{_f(x0)}" y="0" z="0" diameter="{_f(dprox[i])}"/>\n'
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
        w(f'   <channelDensity id="{d.name or f"cd{k}"}" ionChannel="{ch.name}" condDensity="{_f(d.cond)} mS_per_cm2" '
          f'erev="{_f(d.erev)}mV" ion="{ion}"{sg}/>\n')
    w(f'   <spikeThresh value="{_f(c.spike_thresh)}mV"/>\n')
    w(f'   <specificCapacitance value="{_f(c.cm)} uF_per_cm2"/>\n')
    w(f'   <initMembPotential value="{_f(c.v0)}mV"/>\n')
    w('  </membraneProperties>\n  <intracellularProperties>\n')
    w(f'   <resistivity value="{_f(c.ra)} ohm_cm"/>\n')
    w('  </intracellularProperties>\n </biophysicalProperties>\n</cell>\n')


# ---------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------
# unit name -> factor to the NetworkSpec unit of its dimension (mV, ms, nS,
# nA, pF, mS/cm2, uF/cm2, ohm*cm, Hz, per_ms, nS/mV), following the scales
# the reference accepts (eden/NeuroML.cpp:307-400)
_UNITS = {
    "voltage": {"V": 1e3, "mV": 1.0},
    "time": {"s": 1e3, "sec": 1e3, "second": 1e3, "seconds": 1e3, "ms": 1.0, "msec": 1.0, "us": 1e-3,
             "usec": 1e-3},
    "conductance": {"S": 1e9, "mS": 1e6, "uS": 1e3, "nS": 1.0, "pS": 1e-3},
    "current": {"A": 1e9, "mA": 1e6, "uA": 1e3, "nA": 1.0, "pA": 1e-3},
    "capacitance": {"F": 1e12, "mF": 1e9, "uF": 1e6, "nF": 1e3, "pF": 1.0},
    "conductivity": {"S_per_m2": 0.1, "mS_per_cm2": 1.0, "S_per_cm2": 1e3, "S_per_mm2": 1e5},
    "spec_capacitance": {"uF_per_cm2": 1.0, "F_per_m2": 100.0, "uF_per_mm2": 100.0},
    "resistivity": {"ohm_cm": 1.0, "kohm_cm": 1e3, "ohm_m": 100.0},
    "frequency_hz": {"Hz": 1.0, "per_s": 1.0, "per_ms": 1e3, "kHz": 1e3, "per_us": 1e6, "MHz": 1e6},
    "rate_per_ms": {"per_ms": 1.0, "kHz": 1.0, "per_s": 1e-3, "Hz": 1e-3, "per_us": 1e3, "MHz": 1e3},
    "concentration": {"mM": 1.0, "mol_per_cm3": 1e6, "M": 1e3, "uM": 1e-3},
    "resistance": {"ohm": 1e-6, "kohm": 1e-3, "Mohm": 1.0, "Gohm": 1e3},
    "cond_per_voltage": {"nS_per_mV": 1.0, "S_per_V": 1e9 / 1e3, "uS_per_mV": 1e3, "pS_per_mV": 1e-3},
}
_QTY = re.compile(r"^\s*([-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?)\s*([A-Za-z_0-9]*)\s*$")


# PyNN synapse element -> (kind, conductance-based)
_PYNN_SYNAPSES = {"expCondSynapse": (SYN_EXPONE, True), "alphaCondSynapse": (SYN_ALPHA, True),
                  "expCurrSynapse": (SYN_EXPONE_CURRENT, False), "alphaCurrSynapse": (SYN_ALPHA_CURRENT, False)}


def _qty(el, attr, dim, default=None):
    text = el.get(attr)
    if text is None:
        if default is not None:
            return default
        raise ValueError(f"<{_tag(el)}> lacks required attribute {attr}")
    m = _QTY.match(text)
    if not m:
        raise ValueError(f"<{_tag(el)}> {attr}={text!r} is not a number with a unit")
    value, unit = float(m.group(1)), m.group(2)
    if dim is None:
        if unit:
            raise ValueError(f"<{_tag(el)}> {attr}={text!r} should be dimensionless")
        return value
    table = _UNITS[dim]
    if unit not in table:
        raise ValueError(f"<{_tag(el)}> {attr}: unit {unit!r} not supported for {dim} (known: {sorted(table)})")
    return value * table[unit]


def _clamp_key(cl, i):
    side = (lambda x: float(x)) if cl.triple else (lambda x: None)   # a voltageClamp has no before/after targets
    return (cl.triple, float(cl.delay[i]), float(cl.duration[i]), side(cl.v_before[i]), float(cl.v_during[i]),
            side(cl.v_after[i]), float(cl.resistance[i]))


def _wave_key(wv, i):
    return (wv.shape + ("DL" if wv.dimensionless else ""), float(wv.delay[i]), float(wv.duration[i]), float(wv.p0[i]), float(wv.p1[i]),
            float(wv.p2[i]))


def _tag(el):
    return el.tag.split("}")[-1]


def _children(el, tag):
    return [c for c in el if _tag(c) == tag]


_RATE_KIND = {v: k for k, v in RATE_TYPE_NAMES.items()}


_GATE_TAGS = {"rates": "gateHHrates", "tauInf": "gateHHtauInf", "ratesTau": "gateHHratesTau",
              "ratesInf": "gateHHratesInf", "ratesTauInf": "gateHHratesTauInf",
              "instantaneous": "gateHHInstantaneous"}
_GATE_KINDS = {v: k for k, v in _GATE_TAGS.items()}
_VARIABLE_KIND = {"HHExpVariable": 0, "HHExpLinearVariable": 1, "HHSigmoidVariable": 2}
_VARIABLE_TYPE_NAMES = {v: k for k, v in _VARIABLE_KIND.items()}


def _parse_variable(el):
    kind = el.get("type")
    if kind not in _VARIABLE_KIND:
        raise ValueError(f"steadyState type {kind!r} not supported ({', '.join(_VARIABLE_KIND)})")
    return Rate(_VARIABLE_KIND[kind], _qty(el, "rate", None), _qty(el, "midpoint", "voltage"),
                _qty(el, "scale", "voltage"))


def _temperature_degc(text):
    m = _QTY.match(text or "")
    if not m or m.group(2) not in ("degC", "K"):
        raise ValueError(f"temperature {text!r}: a number in degC or K is required")
    value = float(m.group(1))
    return value - 273.15 if m.group(2) == "K" else value


def _parse_rate(el):
    kind = el.get("type")
    if kind not in _RATE_KIND:
        raise ValueError(f"gate rate type {kind!r} not supported (HHExpRate, HHExpLinearRate, HHSigmoidRate)")
    return Rate(_RATE_KIND[kind], _qty(el, "rate", "rate_per_ms"), _qty(el, "midpoint", "voltage"),
                _qty(el, "scale", "voltage"))


def _parse_cell(el, channels_by_name, top=None):
    """A <cell>; its morphology and biophysicalProperties inline or, by the
    cell's attributes of those names, top-level elements of `top` (id ->
    element)."""
    name = el.get("id")
    top = top or {}
    morph = _children(el, "morphology")
    if not morph and el.get("morphology") in top:
        morph = [top[el.get("morphology")]]
    if len(morph) != 1:
        raise ValueError(f"cell {name}: exactly one <morphology> is supported")
    segs = _children(morph[0], "segment")
    ids = [int(s.get("id")) for s in segs]
    index = {sid: i for i, sid in enumerate(ids)}
    n = len(segs)
    parent = np.full(n, -1, np.int64)
    length = np.zeros(n)
    dprox = np.zeros(n)
    ddist = np.zeros(n)
    dist_pt = [None] * n
    for i, s in enumerate(segs):
        par = _children(s, "parent")
        if par:
            if par[0].get("fractionAlong", "1") not in ("1", "1.0"):
                raise ValueError(f"cell {name}: segment {ids[i]} attaches with fractionAlong != 1")
            parent[i] = index[int(par[0].get("segment"))]
            if parent[i] >= i:
                raise ValueError(f"cell {name}: segment {ids[i]} must follow its parent")
        d = _children(s, "distal")[0]
        pr = _children(s, "proximal")
        p_el = pr[0] if pr else None
        dp = np.array([float(d.get(k)) for k in "xyz"])
        if p_el is not None:
            pp = np.array([float(p_el.get(k)) for k in "xyz"])
            dprox[i] = float(p_el.get("diameter"))
        else:
            if parent[i] < 0:
                raise ValueError(f"cell {name}: root segment needs a proximal point")
            pp = dist_pt[parent[i]]
            dprox[i] = ddist[parent[i]]
        ddist[i] = float(d.get("diameter"))
        dist_pt[i] = dp
        length[i] = float(np.sqrt(((dp - pp) ** 2).sum()))
    if ids != sorted(ids) or ids[0] != 0:
        raise ValueError(f"cell {name}: segments must be numbered 0.. in order")
    groups = {}
    for g in _children(morph[0], "segmentGroup"):
        mask = np.zeros(n, bool)
        for mbr in _children(g, "member"):
            mask[index[int(mbr.get("segment"))]] = True
        for inc in _children(g, "include"):
            mask |= groups[inc.get("segmentGroup")]
        if _children(g, "property"):
            raise ValueError(f"cell {name}: segment group properties (cable subdivision) are not supported")
        groups[g.get("id")] = mask
    groups.setdefault("all", np.ones(n, bool))
    bio = _children(el, "biophysicalProperties")
    if not bio and el.get("biophysicalProperties") in top:
        bio = [top[el.get("biophysicalProperties")]]
    if len(bio) != 1:
        raise ValueError(f"cell {name}: exactly one <biophysicalProperties> is supported")
    bio = bio[0]
    mem = _children(bio, "membraneProperties")[0]
    intra = _children(bio, "intracellularProperties")[0]
    dens = []
    cm = v0 = thr = None
    for c in mem:
        t = _tag(c)
        if t == "channelDensity":
            ch = c.get("ionChannel")
            if ch not in channels_by_name:
                raise ValueError(f"cell {name}: unknown ionChannel {ch}")
            mask = groups[c.get("segmentGroup", "all")]
            dens.append(ChannelDensity(channels_by_name[ch], _qty(c, "condDensity", "conductivity"),
                                       _qty(c, "erev", "voltage"), mask.copy(), c.get("id", "")))
        elif t == "specificCapacitance":
            cm = _qty(c, "value", "spec_capacitance")
        elif t == "initMembPotential":
            v0 = _qty(c, "value", "voltage")
        elif t == "spikeThresh":
            thr = _qty(c, "value", "voltage")
        else:
            raise ValueError(f"cell {name}: <{t}> is not supported")
    ra = _qty(_children(intra, "resistivity")[0], "value", "resistivity")
    cell = PhysicalCell(name, parent, length, ddist.copy(), dens, cm=cm, ra=ra, v0=v0,
                        spike_thresh=thr if thr is not None else 0.0, seg_groups=groups,
                        seg_dprox=None if np.array_equal(dprox, ddist) else dprox.copy())
    return cell


def read_event_set(path: str, instances: int, ports: int) -> list:
    """An event-set file in EDEN's ascii_v0 form: per line a timestamp (s)
    and tokens `instance` or `instance!port` (eden/Eden.cpp:10759-10826)."""
    frames = []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok:
                continue
            pairs = []
            for t in tok[1:]:
                inst, _, port = t.partition("!")
                i, p_ = int(inst), int(port or 0)
                if not (0 <= i < instances and 0 <= p_ < ports):
                    raise ValueError(f"{path}: event {t!r} out of range")
                pairs.append((i, p_))
            frames.append((float(tok[0]), pairs))
    return frames


def _cell_ref(text, pops, default_pop=None):
    """'../pop[3]', '../pop/3/celltype', 'pop[3]', 'pop/3', or a bare index
    ('3' or '/3') of the projection's population -> (population, index)."""
    t = text.strip()
    if default_pop is not None and re.fullmatch(r"/?\d+", t):
        return default_pop, int(t.lstrip("/"))
    while t.startswith("../"):
        t = t[3:]
    m = re.match(r"^([^/\[\]]+)\[(\d+)\]", t)
    if m:
        return m.group(1), int(m.group(2))
    parts = t.split("/")
    if len(parts) >= 2 and parts[0] in pops:
        return parts[0], int(parts[1])
    raise ValueError(f"cell reference {text!r} not understood")


def read_lems(path: str) -> NetworkSpec:
    """Read a LEMS simulation file (and the NeuroML it includes) into a
    NetworkSpec.  Raises ValueError on anything outside the supported subset."""
    base = os.path.dirname(os.path.abspath(path))
    root = ET.parse(path).getroot()
    elems = list(root)
    for inc in _children(root, "Include"):
        f = inc.get("file")
        if f in ("Cells.xml", "Networks.xml", "Simulation.xml", "Synapses.xml", "Inputs.xml",
                 "NeuroMLCoreDimensions.xml", "NeuroMLCoreCompTypes.xml", "Channels.xml", "PyNN.xml"):
            continue
        fp = os.path.join(base, f)
        elems.extend(list(ET.parse(fp).getroot()))
    target = _children(root, "Target")[0].get("component")
    sims = [e for e in elems if _tag(e) == "Simulation" and e.get("id") == target]
    if not sims:
        raise ValueError(f"simulation {target} not found")
    sim = sims[0]
    seed = int(sim.get("seed", "0"))
    spec = NetworkSpec(os.path.splitext(os.path.basename(path))[0], _qty(sim, "step", "time"),
                       _qty(sim, "length", "time"), seed)
    # components
    channels_by_name, synapses, pulses_def, pois_def, cells = {}, {}, {}, {}, {}
    timed_def, wave_def, clamp_def, gap_def = {}, {}, {}, {}
    refused_inputs = {}
    net = None
    # morphologies and biophysical properties a cell may name by id
    top_parts = {e.get("id"): e for e in elems if _tag(e) in ("morphology", "biophysicalProperties")}
    for e in elems:
        t = _tag(e)
        if t == "ionChannelHH" or t == "ionChannel":
            gates = []
            for g in e:
                gt = _tag(g)
                if gt in ("notes", "annotation"):
                    continue
                if gt not in _GATE_KINDS:
                    raise ValueError(f"ionChannel {e.get('id')}: <{gt}> not supported "
                                     f"({', '.join(sorted(_GATE_KINDS))})")
                kind = _GATE_KINDS[gt]
                fwd = rev = tau = inf = q10 = None
                if kind not in ("tauInf", "instantaneous"):
                    fwd = _parse_rate(_children(g, "forwardRate")[0])
                    rev = _parse_rate(_children(g, "reverseRate")[0])
                if kind in ("tauInf", "ratesTau", "ratesTauInf"):
                    tc = _children(g, "timeCourse")[0]
                    if tc.get("type") != "fixedTimeCourse":
                        raise ValueError(f"ionChannel {e.get('id')} gate {g.get('id')}: timeCourse type "
                                         f"{tc.get('type')!r} not supported (fixedTimeCourse)")
                    tau = _qty(tc, "tau", "time")
                if kind in ("tauInf", "ratesInf", "ratesTauInf", "instantaneous"):
                    inf = _parse_variable(_children(g, "steadyState")[0])
                for qs in _children(g, "q10Settings"):
                    if qs.get("type") == "q10Fixed":
                        q10 = ("fixed", _qty(qs, "fixedQ10", None))
                    elif qs.get("type") == "q10ExpTemp":
                        q10 = ("exp", _qty(qs, "q10Factor", None), _temperature_degc(qs.get("experimentalTemp")))
                    else:
                        raise ValueError(f"q10Settings type {qs.get('type')!r} not supported")
                gates.append(Gate(g.get("id"), int(g.get("instances", "1")), fwd, rev, kind, tau, inf, q10))
            channels_by_name[e.get("id")] = len(spec.channels)
            spec.channels.append(Channel(e.get("id"), gates, e.get("species")))
        elif t == "expOneSynapse":
            synapses[e.get("id")] = SynapseType(e.get("id"), SYN_EXPONE, _qty(e, "gbase", "conductance"),
                                                _qty(e, "erev", "voltage"), _qty(e, "tauDecay", "time"))
        elif t == "expTwoSynapse":
            synapses[e.get("id")] = SynapseType(e.get("id"), SYN_EXPTWO, _qty(e, "gbase", "conductance"),
                                                _qty(e, "erev", "voltage"), _qty(e, "tauDecay", "time"),
                                                _qty(e, "tauRise", "time"))
        elif t == "alphaSynapse":
            synapses[e.get("id")] = SynapseType(e.get("id"), SYN_ALPHA, _qty(e, "gbase", "conductance"),
                                                _qty(e, "erev", "voltage"), _qty(e, "tau", "time"))
        elif t == "alphaCurrentSynapse":
            synapses[e.get("id")] = SynapseType(e.get("id"), SYN_ALPHA_CURRENT, _qty(e, "ibase", "current"), 0.0,
                                                _qty(e, "tau", "time"))
        elif t == "blockingPlasticSynapse":
            # LEMS_CoreComponents.inc.xml:315-352, with at most one block
            # mechanism (voltageConcDepBlockMechanism, 231-245) and one
            # plasticity mechanism (tsodyksMarkram(DepFac)Mechanism, 247-312)
            block = plast = None
            for ch in e:
                ct = _tag(ch)
                if ct == "blockMechanism":
                    if ch.get("type") != "voltageConcDepBlockMechanism":
                        raise ValueError(f"{e.get('id')}: block mechanism {ch.get('type')!r} not supported")
                    block = {"blockConcentration": _qty(ch, "blockConcentration", "concentration"),
                             "scalingConc": _qty(ch, "scalingConc", "concentration"),
                             "scalingVolt": _qty(ch, "scalingVolt", "voltage"), "species": ch.get("species", "")}
                elif ct == "plasticityMechanism":
                    kind = ch.get("type")
                    if kind not in ("tsodyksMarkramDepMechanism", "tsodyksMarkramDepFacMechanism"):
                        raise ValueError(f"{e.get('id')}: plasticity mechanism {kind!r} not supported")
                    plast = {"type": kind, "initReleaseProb": _qty(ch, "initReleaseProb", None),
                             "tauRec": _qty(ch, "tauRec", "time")}
                    if kind.endswith("DepFacMechanism"):
                        plast["tauFac"] = _qty(ch, "tauFac", "time")
            synapses[e.get("id")] = SynapseType(e.get("id"), SYN_BLOCKING_PLASTIC, _qty(e, "gbase", "conductance"),
                                                _qty(e, "erev", "voltage"), _qty(e, "tauDecay", "time"),
                                                _qty(e, "tauRise", "time"), block=block, plasticity=plast)
        elif t == "expThreeSynapse":
            synapses[e.get("id")] = SynapseType(e.get("id"), SYN_EXPTHREE, _qty(e, "gbase1", "conductance"),
                                                _qty(e, "erev", "voltage"), _qty(e, "tauDecay1", "time"),
                                                _qty(e, "tauRise", "time"), _qty(e, "gbase2", "conductance"),
                                                _qty(e, "tauDecay2", "time"))
        elif t in _PYNN_SYNAPSES:
            # PyNN synapses (LEMS_CoreComponents.inc.xml:1834-1940): tau_syn in
            # ms and e_rev in mV, without units; the state jumps by the
            # weight property (1) and is a conductance in uS or a current in nA
            kind, cond = _PYNN_SYNAPSES[t]
            synapses[e.get("id")] = SynapseType(e.get("id"), kind, 1000.0 if cond else 1.0,
                                                _qty(e, "e_rev", None) if cond else 0.0, _qty(e, "tau_syn", None),
                                                form=t)
        elif t in ("gapJunction", "linearGradedSynapse"):
            gap_def[e.get("id")] = GapJunctionType(e.get("id"), _qty(e, "conductance", "conductance"), kind=t)
        elif t == "silentSynapse":
            gap_def[e.get("id")] = GapJunctionType(e.get("id"), 0.0, kind=t)
        elif t == "gradedSynapse":
            # LEMS_CoreComponents.inc.xml:38-80
            gap_def[e.get("id")] = GapJunctionType(e.get("id"), _qty(e, "conductance", "conductance"), kind=t,
                                                   delta=_qty(e, "delta", "voltage"), k=_qty(e, "k", "rate_per_ms"),
                                                   vth=_qty(e, "Vth", "voltage"), erev=_qty(e, "erev", "voltage"))
        elif t in ("pulseGenerator", "pulseGeneratorDL"):
            dl = t.endswith("DL")
            pulses_def[e.get("id")] = (_qty(e, "delay", "time"), _qty(e, "duration", "time"),
                                       _qty(e, "amplitude", None if dl else "current"), dl)
        elif t == "fitzHughNagumoCell":
            cells[e.get("id")] = FitzHughNagumoCell(e.get("id"), _qty(e, "I", None))
        elif t == "izhikevichCell":
            cells[e.get("id")] = IzhikevichCell(e.get("id"), _qty(e, "v0", "voltage"), _qty(e, "thresh", "voltage"),
                                                _qty(e, "a", None), _qty(e, "b", None), _qty(e, "c", None),
                                                _qty(e, "d", None))
        elif t == "timedSynapticInput":
            timed_def[e.get("id")] = (e.get("synapse"), [_qty(sp, "time", "time") for sp in _children(e, "spike")])
        elif t == "poissonFiringSynapse":
            pois_def[e.get("id")] = (_qty(e, "averageRate", "frequency_hz"), e.get("synapse"))
        elif t == "transientPoissonFiringSynapse":
            # the reference writes this component's LONG_TIME constant (1e9
            # hour) as `inf` into its generated C, which then fails to compile:
            # refused where an input list uses it (a definition alone is fine)
            refused_inputs[e.get("id")] = (f"transientPoissonFiringSynapse {e.get('id')}: not supported (the "
                                           f"reference simulator cannot run it either)")
        elif t in ("voltageClamp", "voltageClampTriple"):
            if e.get("simpleSeriesResistance") is not None:
                res = _qty(e, "simpleSeriesResistance", "resistance")
            else:   # the reference scales the older attribute by 1e5 (eden/NeuroML.cpp:7091-7100)
                res = _qty(e, "seriesResistance", "resistance") * 1e5
            if t == "voltageClamp":
                v = _qty(e, "targetVoltage", "voltage")
                clamp_def[e.get("id")] = (False, _qty(e, "delay", "time"), _qty(e, "duration", "time"),
                                          np.nan, v, np.nan, res)
            else:
                if _qty(e, "active", None) != 1.0:
                    raise ValueError(f"voltageClampTriple {e.get('id')}: only active=\"1\" is supported")
                clamp_def[e.get("id")] = (True, _qty(e, "delay", "time"), _qty(e, "duration", "time"),
                                          _qty(e, "conditioningVoltage", "voltage"),
                                          _qty(e, "testingVoltage", "voltage"), _qty(e, "returnVoltage", "voltage"),
                                          res)
        elif t in ("sineGenerator", "sineGeneratorDL"):
            cur = None if t.endswith("DL") else "current"
            wave_def[e.get("id")] = (WAVE_SINE, _qty(e, "delay", "time"), _qty(e, "duration", "time"),
                                     _qty(e, "amplitude", cur), _qty(e, "period", "time"),
                                     _qty(e, "phase", None), cur is None)
        elif t in ("rampGenerator", "rampGeneratorDL"):
            cur = None if t.endswith("DL") else "current"
            wave_def[e.get("id")] = (WAVE_RAMP, _qty(e, "delay", "time"), _qty(e, "duration", "time"),
                                     _qty(e, "startAmplitude", cur), _qty(e, "finishAmplitude", cur),
                                     _qty(e, "baselineAmplitude", cur), cur is None)
        elif t == "izhikevich2007Cell":
            cells[e.get("id")] = Izhikevich2007Cell(
                e.get("id"), C=_qty(e, "C", "capacitance"), k=_qty(e, "k", "cond_per_voltage"),
                vr=_qty(e, "vr", "voltage"), vt=_qty(e, "vt", "voltage"), vpeak=_qty(e, "vpeak", "voltage"),
                a=_qty(e, "a", "rate_per_ms"), b=_qty(e, "b", "conductance"), c=_qty(e, "c", "voltage"),
                d=_qty(e, "d", "current") * 1e3, v0=_qty(e, "v0", "voltage"))  # d in pA
        elif t in ("iafTauCell", "iafTauRefCell", "iafCell", "iafRefCell"):
            tau_kind = t.startswith("iafTau")
            cells[e.get("id")] = IafCell(
                e.get("id"), t, _qty(e, "leakReversal", "voltage"), _qty(e, "thresh", "voltage"),
                _qty(e, "reset", "voltage"),
                tau=_qty(e, "tau", "time") if tau_kind else 0.0,
                C=0.0 if tau_kind else _qty(e, "C", "capacitance"),
                leak_conductance=0.0 if tau_kind else _qty(e, "leakConductance", "conductance"),
                refract=_qty(e, "refract", "time") if t.endswith("RefCell") else 0.0)
        elif t == "adExIaFCell":
            cells[e.get("id")] = AdExCell(
                e.get("id"), C=_qty(e, "C", "capacitance"), gL=_qty(e, "gL", "conductance"),
                EL=_qty(e, "EL", "voltage"), VT=_qty(e, "VT", "voltage"), thresh=_qty(e, "thresh", "voltage"),
                reset=_qty(e, "reset", "voltage"), delT=_qty(e, "delT", "voltage"), tauw=_qty(e, "tauw", "time"),
                refract=_qty(e, "refract", "time"), a=_qty(e, "a", "conductance"), b=_qty(e, "b", "current"))
        elif t == "spikeArray":
            cells[e.get("id")] = SpikeArrayCell(e.get("id"),
                                                np.array([_qty(sp, "time", "time") for sp in _children(e, "spike")]))
        elif t == "spikeGenerator":
            cells[e.get("id")] = SpikeGeneratorCell(e.get("id"), _qty(e, "period", "time"))
        elif t == "spikeGeneratorRandom":
            cells[e.get("id")] = SpikeGeneratorRandomCell(e.get("id"), _qty(e, "minISI", "time"),
                                                          _qty(e, "maxISI", "time"))
        elif t == "spikeGeneratorPoisson":
            cells[e.get("id")] = SpikeGeneratorPoissonCell(e.get("id"), _qty(e, "averageRate", "frequency_hz"))
        elif t == "spikeGeneratorRefPoisson":
            cells[e.get("id")] = SpikeGeneratorPoissonCell(e.get("id"), _qty(e, "averageRate", "frequency_hz"),
                                                           _qty(e, "minimumISI", "time"))
        elif t in ("network", "networkWithTemperature") and e.get("id") == sim.get("target"):
            net = e
    for e in elems:
        if _tag(e) == "cell":
            cells[e.get("id")] = _parse_cell(e, channels_by_name, top_parts)
    if net is None:
        raise ValueError(f"network {sim.get('target')} not found")
    if _tag(net) == "networkWithTemperature" or net.get("type") == "networkWithTemperature":
        spec.temperature = _temperature_degc(net.get("temperature"))
    spec.synapses = list(synapses.values())
    spec.gap_types = list(gap_def.values())
    syn_names = list(synapses)
    # network elements that carry dynamics and are not read fail loudly
    # rather than drop out of the simulation
    for el in net:
        if _tag(el) in ("EdenTimeSeriesReader", "cellSet", "synapticConnection"):
            raise ValueError(f"<{_tag(el)} id={el.get('id')}> is not supported")
    # populations (declaration order = gid order)
    pops = {}
    for p in _children(net, "population"):
        comp = p.get("component")
        if comp not in cells:
            raise ValueError(f"population {p.get('id')}: component {comp} not supported")
        size = int(p.get("size")) if p.get("size") else len(_children(p, "instance"))
        pops[p.get("id")] = Population(p.get("id"), comp, size)
        spec.populations.append(pops[p.get("id")])
    # EDEN's event-set readers (eden/NeuroML.cpp:6455-6495): their sources
    # follow the cells in global order, as they are no work items
    readers = {}
    for r in _children(net, "EdenEventSetReader"):
        if r.get("format") != "ascii_v0":
            raise ValueError(f"EdenEventSetReader {r.get('id')}: format {r.get('format')!r} not supported")
        href = r.get("href") or ""
        if href.startswith("file://"):
            href = href[len("file://"):]
        fpath = os.path.join(base, href)
        if not os.path.isfile(fpath):
            raise ValueError(f"EdenEventSetReader {r.get('id')}: {href} is not a readable file")
        ports = [pt.get("id") for pt in _children(r, "Port")]
        n_inst = int(r.get("instances"))
        cell = EventSetReaderCell(r.get("id"), n_inst, ports, read_event_set(fpath, n_inst, len(ports)),
                                  href=os.path.basename(href))
        cells[cell.name] = cell
        readers[cell.name] = cell
        pops[cell.name] = Population(cell.name, cell.name, n_inst * len(ports))
        spec.populations.append(pops[cell.name])
    used = {p.cell_type for p in spec.populations}
    spec.cells = [c for n_, c in cells.items() if n_ in used]
    off = spec.pop_offsets()
    gid = lambda pop_idx: off[pop_idx[0]] + pop_idx[1]

    def pre_gid(c, pr):
        # a connection's presynaptic source; an event-set reader's is its
        # (instance, port), the port named by preSegmentId
        pop = pr.get("presynapticPopulation")
        if pop in readers:
            ports = readers[pop].ports
            seg = c.get("preSegmentId")
            port = ports.index(seg) if seg in ports else int(seg or 0)
            return off[pop] + int(c.get("preCellId")) * len(ports) + port
        return gid(_cell_ref(c.get("preCellId"), pops, pop))
    # projections
    by_syn = {}
    for pr in _children(net, "projection"):
        syn = pr.get("synapse")
        if syn not in synapses:
            raise ValueError(f"projection {pr.get('id')}: synapse {syn} not supported")
        rows = by_syn.setdefault(syn, [[], [], [], [], [], []])
        for c in pr:
            if _tag(c) not in ("connectionWD", "connection"):
                continue
            rows[5].append((pr.get("id"), int(c.get("id"))))
            rows[0].append(pre_gid(c, pr))
            rows[1].append(gid(_cell_ref(c.get("postCellId"), pops, pr.get("postsynapticPopulation"))))
            rows[2].append(int(c.get("postSegmentId", "0")))
            rows[3].append(float(c.get("weight", "1")))
            rows[4].append(_qty(c, "delay", "time", 0.0) if c.get("delay") else 0.0)
    for syn, rows in by_syn.items():
        spec.projections.append(Projection(f"proj_{syn}", "*", "*", syn, np.array(rows[0], np.int64),
                                           np.array(rows[1], np.int64), np.array(rows[2], np.int64),
                                           np.array(rows[3]), np.array(rows[4]), conn_ids=rows[5]))
    # electrical projections: gap junctions, an instance on each end
    # (eden/NeuroML.cpp:6057-6125: electricalConnection with cell indices,
    # electricalConnectionInstance(W) with cell paths, W with a weight)
    by_gap = {}
    for pr in _children(net, "electricalProjection"):
        pa, pb = pr.get("presynapticPopulation"), pr.get("postsynapticPopulation")
        for c in pr:
            tag = _tag(c)
            if tag not in ("electricalConnection", "electricalConnectionInstance", "electricalConnectionInstanceW"):
                continue
            syn = c.get("synapse")
            if syn not in gap_def:
                raise ValueError(f"electricalProjection {pr.get('id')}: synapse {syn} is not a gapJunction, "
                                 f"linearGradedSynapse, gradedSynapse or silentSynapse")
            rows = by_gap.setdefault(syn, [[], [], [], [], []])
            rows[0].append(gid(_cell_ref(c.get("preCell"), pops, pa)))
            rows[1].append(int(c.get("preSegment", "0")))
            rows[2].append(gid(_cell_ref(c.get("postCell"), pops, pb)))
            rows[3].append(int(c.get("postSegment", "0")))
            rows[4].append(float(c.get("weight", "1")) if tag.endswith("W") else 1.0)
    for syn, rows in by_gap.items():
        spec.electrical.append(ElectricalProjection(f"gap_{syn}", syn, *(np.array(r, np.int64) for r in rows[:4]),
                                                    np.array(rows[4])))
    # continuous projections: preComponent on the pre end, postComponent on
    # the post end (eden/NeuroML.cpp:6126-6128 the connection forms,
    # 6243-6260 the components; eden/Eden.cpp:9254-9270 both ends)
    for pr in _children(net, "continuousProjection"):
        pa, pb = pr.get("presynapticPopulation"), pr.get("postsynapticPopulation")
        by_pair = {}
        for c in pr:
            tag = _tag(c)
            if tag not in ("continuousConnection", "continuousConnectionInstance", "continuousConnectionInstanceW"):
                continue
            key = (c.get("preComponent"), c.get("postComponent"))
            for comp in key:
                if comp not in gap_def:
                    raise ValueError(f"continuousProjection {pr.get('id')}: component {comp} is not a "
                                     f"linearGradedSynapse, gradedSynapse, silentSynapse or gapJunction")
            rows = by_pair.setdefault(key, [[], [], [], [], []])
            rows[0].append(gid(_cell_ref(c.get("preCell"), pops, pa)))
            rows[1].append(int(c.get("preSegment", "0")))
            rows[2].append(gid(_cell_ref(c.get("postCell"), pops, pb)))
            rows[3].append(int(c.get("postSegment", "0")))
            rows[4].append(float(c.get("weight", "1")) if tag.endswith("W") else 1.0)
        for (ca, cb), rows in by_pair.items():
            spec.continuous.append(ContinuousProjection(pr.get("id"), ca, cb,
                                                        *(np.array(r, np.int64) for r in rows[:4]),
                                                        np.array(rows[4])))
    # inputs
    pcell, pseg, pdel, pdur, pamp, pwt, pdl, plist = [], [], [], [], [], [], [], []
    pois_rows, wave_rows, clamp_rows = {}, {}, {}
    timed_rows = {}
    for il in _children(net, "inputList"):
        comp = il.get("component")
        for inp in _children(il, "input") + _children(il, "inputW"):
            g = gid(_cell_ref(inp.get("target"), pops, il.get("population")))
            seg = int(inp.get("segmentId", "0"))
            if comp in timed_def:
                timed_rows.setdefault(timed_def[comp][0], []).append(
                    (g, seg, timed_def[comp][1], float(inp.get("weight", "1"))))
            elif comp in pulses_def:
                d, du, a, dl = pulses_def[comp]
                pcell.append(g); pseg.append(seg); pdel.append(d); pdur.append(du); pamp.append(a)
                pwt.append(float(inp.get("weight", "1"))); pdl.append(dl)
                plist.append((il.get("id"), int(inp.get("id"))))
            elif comp in pois_def:
                pois_rows.setdefault(comp, []).append((g, seg))
            elif comp in wave_def:
                wave_rows.setdefault(comp, []).append((g, seg, float(inp.get("weight", "1")),
                                                       (il.get("id"), int(inp.get("id")))))
            elif comp in clamp_def:
                clamp_rows.setdefault(comp, []).append((g, seg, float(inp.get("weight", "1")),
                                                        (il.get("id"), int(inp.get("id")))))
            elif comp in refused_inputs:
                raise ValueError(refused_inputs[comp])
            else:
                raise ValueError(f"inputList component {comp} not supported")
    for ei in _children(net, "explicitInput"):
        comp = ei.get("input")
        g = gid(_cell_ref(ei.get("target"), pops))
        if comp not in pulses_def:
            raise ValueError(f"explicitInput {comp} not supported")
        d, du, a, dl = pulses_def[comp]
        pcell.append(g); pseg.append(0); pdel.append(d); pdur.append(du); pamp.append(a); pwt.append(1.0)
        pdl.append(dl); plist.append(None)
    for dl in (False, True):
        sel = [i for i in range(len(pcell)) if pdl[i] == dl]
        if not sel:
            continue
        pick = lambda xs: np.array([xs[i] for i in sel])
        wts = pick(pwt)
        lids = [plist[i] for i in sel]
        spec.pulses.append(PulseInputs("*", pick(pcell), pick(pseg), pick(pdel), pick(pdur), pick(pamp),
                                       None if (wts == 1.0).all() else wts, dl,
                                       None if any(x is None for x in lids) else lids))
    for syn, rows in timed_rows.items():
        if syn not in synapses:
            raise ValueError(f"timedSynapticInput: synapse {syn} not supported")
        spec.timed.append(TimedInputs(syn, np.array([r[0] for r in rows], np.int64),
                                      np.array([r[1] for r in rows], np.int64), [np.array(r[2]) for r in rows],
                                      np.array([r[3] for r in rows])))
    # Poisson components in the order they are defined (the reference numbers
    # their random draws in that order)
    for comp, (rate, syn) in pois_def.items():
        rows = pois_rows.get(comp)
        if not rows:
            continue
        if syn not in synapses:
            raise ValueError(f"poissonFiringSynapse {comp}: synapse {syn} not supported")
        spec.poissons.append(PoissonInputs("*", syn, rate, np.array([r[0] for r in rows]),
                                           np.array([r[1] for r in rows])))
    for comp, rows in clamp_rows.items():
        triple, d, du, vb, vd, va, res = clamp_def[comp]
        n = len(rows)
        spec.clamps.append(ClampInputs(triple, np.array([r[0] for r in rows], np.int64),
                                       np.array([r[1] for r in rows], np.int64), np.full(n, d), np.full(n, du),
                                       np.full(n, vb), np.full(n, vd), np.full(n, va), np.full(n, res),
                                       np.array([r[2] for r in rows]), [r[3] for r in rows]))
    for comp, rows in wave_rows.items():
        shape, d, du, a, b, c, dl = wave_def[comp]
        n = len(rows)
        spec.waves.append(WaveInputs(shape, np.array([r[0] for r in rows], np.int64),
                                     np.array([r[1] for r in rows], np.int64), np.full(n, d), np.full(n, du),
                                     np.full(n, a), np.full(n, b), np.full(n, c),
                                     np.array([r[2] for r in rows]), dl, [r[3] for r in rows]))
    # recorders: OutputFile / EventOutputFile and EDEN's EdenOutputFile /
    # EdenEventOutputFile with their time window, sampling interval or explicit
    # sample points, and heartbeat interval (eden/NeuroML.cpp:8037-8290);
    # times are kept in us
    spec.trace_columns, spec.event_selections = [], []
    spec.output_files, spec.event_files = [], []
    inf = float("inf")

    def _path(e):
        if e.get("fileName") is not None:
            return e.get("fileName")
        href = e.get("href") or ""
        if not href.startswith("file://"):
            raise ValueError(f"<{_tag(e)} id={e.get('id')}>: only file:// outputs are supported")
        return href[len("file://"):]

    def _us(e, attr, default):
        return _qty(e, attr, "time") * 1e3 if e.get(attr) is not None else default

    # recorded membrane potentials leave the engine in mV: classic OutputFile
    # columns are written in SI units, EdenOutputFile columns in their
    # output_units (eden/NeuroML.cpp:8170-8183)
    volt_out = {"V": 1e-3, "mV": 1.0, "uV": 1e3}
    for of in [c for c in sim if _tag(c) in ("OutputFile", "EdenOutputFile")]:
        cols = []
        for col in _children(of, "OutputColumn"):
            units = col.get("output_units") if _tag(of) == "EdenOutputFile" else "V"
            if units not in volt_out:
                raise ValueError(f"OutputColumn {col.get('id')}: output_units {units!r} not supported")
            # a fitzHughNagumoCell's V and a gate's state q are dimensionless:
            # written as they are
            qs = col.get("quantity").strip()
            scale = 1.0 if qs.endswith("/V") or qs.endswith("/q") else volt_out[units]
            cols.append((col.get("id"), col.get("quantity"), _quantity_target(col.get("quantity"), pops, cells),
                         scale))
        points = None
        for sp in _children(of, "SamplePoints"):
            points = [_qty(x, "t", "time") * 1e3 for x in _children(sp, "s")]
        spec.output_files.append({"id": of.get("id"), "path": _path(of), "cols": cols,
                                  "start": _us(of, "starting_from", -inf), "end": _us(of, "up_to_excluding", inf),
                                  "interval": _us(of, "sampling_interval", 0.0), "points": points})
        spec.trace_columns.extend(OutputColumn(*c[2]) for c in cols)
    for ef in [c for c in sim if _tag(c) in ("EventOutputFile", "EdenEventOutputFile")]:
        sels = []
        for sel in _children(ef, "EventSelection"):
            pop, idx = _cell_ref(sel.get("select"), pops)
            sels.append((int(sel.get("id")), sel.get("select"), (pop, idx)))
        fmt = ef.get("format", "TIME_ID")
        if fmt not in ("TIME_ID", "ID_TIME", "ascii_v0"):
            raise ValueError(f"<{_tag(ef)} id={ef.get('id')}>: unknown format {fmt}")
        spec.event_files.append({"id": ef.get("id"), "path": _path(ef), "format": fmt, "sels": sels,
                                 "start": _us(ef, "starting_from", -inf), "end": _us(ef, "up_to_excluding", inf),
                                 "max_interval": _us(ef, "maximum_interval", inf)})
        spec.event_selections.extend(EventSelection(s[2][0], s[2][1], 0) for s in sels)
    for cs in _children(sim, "EdenCustomSetup"):
        from .custom_setup import parse as parse_setup
        with open(os.path.join(os.path.dirname(os.path.abspath(path)), cs.get("filename"))) as f:
            spec.custom_setup += parse_setup(f.read(), spec)
    return spec


def _quantity_target(q, pops, cells):
    """'pop/3/celltype/seg/v', 'pop/3/celltype/v' or 'pop[3]/v' -> (pop, cell,
    seg, "v"); a gate's state, 'pop/3/celltype/seg/<biophysicalProperties
    id>/membraneProperties/<channelDensity id>/<ionChannel id>/<gate id>/q'
    -> (pop, cell, seg, "q:<channelDensity id>/<gate id>")."""
    parts = q.strip().split("/")
    if parts[-1] == "q" and "membraneProperties" in parts:
        i = parts.index("membraneProperties")
        if len(parts) != i + 5:
            raise ValueError(f"recorded quantity {q!r}: expected .../membraneProperties/<channelDensity>/"
                             f"<ionChannel>/<gate>/q")
        pop, cell, seg, _ = _quantity_target("/".join(parts[:i - 1] + ["v"]), pops, cells)
        return (pop, cell, seg, f"q:{parts[i + 1]}/{parts[i + 3]}")
    if parts[-1] not in ("v", "V"):
        raise ValueError(f"recorded quantity {q!r}: only membrane potential v (a fitzHughNagumoCell's V) "
                         f"and gate states q are supported")
    m = re.match(r"^([^/\[\]]+)\[(\d+)\]$", parts[0])
    if m:
        pop, idx, rest = m.group(1), int(m.group(2)), parts[1:-1]
    else:
        pop, idx, rest = parts[0], int(parts[1]), parts[2:-1]
        if rest and rest[0] in cells:
            rest = rest[1:]
    seg = int(rest[0]) if rest else 0
    if pop not in pops:
        raise ValueError(f"recorded quantity {q!r}: unknown population")
    return (pop, idx, seg, "v")
