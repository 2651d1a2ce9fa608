"""EdenCustomSetup files: per-instance overrides of a network's properties.

The reference reads `set` statements from the file an `<EdenCustomSetup
filename=...>` element of the LEMS `<Simulation>` names
(eden/NeuroML.cpp:7240-7330 tokenising, 7629-7790 `set cell`, 7430-7500
values and units) and applies them to the instances' tables before the run
(eden/Eden.cpp:9437-9649):

    set cell <population> <instance ids | all> all <property> <value> <unit>
    set cell <population> <instance ids | all> all <property> multi <unit>
    values <one value per selected instance>

    set input <inputList> <input ids | all> <property> <value | multi> [<unit>]

    set synapse <projection> <connection ids | all> post <property> <value | multi> [<unit>]

Instance ids are comma-separated; a dimensional property needs its unit.
Built here: `set cell` on point neurons (izhikevich2007Cell, iaf*Cell,
adExIaFCell, izhikevichCell), whose LEMS parameters become per-instance
values in the lowered model; `set input` on the pulse, sine, ramp (and
their DL forms) and voltage-clamp inputs of lists read from NeuroML; and
`set synapse` on the postsynaptic component of a projection's connections
(the parameters of its expOne, expTwo, alpha or alphaCurrent synapse,
eden/NeuroML.cpp:7853-7960), where each distinct set of overridden values
becomes a synapse type of its own in the lowered model.  Properties of
physical cells (segment voltage, gate states, calcium) are refused by
name, as the reference refuses them when it applies the setup (its
`set cell` application takes artificial-cell parameters only,
eden/Eden.cpp:9501-9553).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional

import copy

import numpy as np

from .network import (SYN_ALPHA, SYN_ALPHA_CURRENT, SYN_EXPTHREE, SYN_EXPTWO, WAVE_SINE, AdExCell, IafCell, Izhikevich2007Cell,
                      IzhikevichCell)

# LEMS parameter -> (dataclass field, dimension of the unit table, factor to the field's unit)
_IZH = {"v0": ("v0", "voltage", 1.0), "C": ("C", "capacitance", 1.0), "k": ("k", "cond_per_voltage", 1.0),
        "vr": ("vr", "voltage", 1.0), "vt": ("vt", "voltage", 1.0), "vpeak": ("vpeak", "voltage", 1.0),
        "a": ("a", "rate_per_ms", 1.0), "b": ("b", "conductance", 1.0), "c": ("c", "voltage", 1.0),
        "d": ("d", "current", 1e3)}
_IAF = {"leakReversal": ("leak_reversal", "voltage", 1.0), "thresh": ("thresh", "voltage", 1.0),
        "reset": ("reset", "voltage", 1.0), "tau": ("tau", "time", 1.0), "C": ("C", "capacitance", 1.0),
        "leakConductance": ("leak_conductance", "conductance", 1.0), "refract": ("refract", "time", 1.0)}
_ADEX = {"C": ("C", "capacitance", 1.0), "gL": ("gL", "conductance", 1.0), "EL": ("EL", "voltage", 1.0),
         "VT": ("VT", "voltage", 1.0), "thresh": ("thresh", "voltage", 1.0), "reset": ("reset", "voltage", 1.0),
         "delT": ("delT", "voltage", 1.0), "tauw": ("tauw", "time", 1.0), "refract": ("refract", "time", 1.0),
         "a": ("a", "conductance", 1.0), "b": ("b", "current", 1.0)}


_IZH_DL = {"v0": ("v0", "voltage", 1.0), "thresh": ("thresh", "voltage", 1.0), "a": ("a", None, 1.0),
           "b": ("b", None, 1.0), "c": ("c", None, 1.0), "d": ("d", None, 1.0)}


def _params_of(ct):
    if isinstance(ct, IzhikevichCell):
        return _IZH_DL
    if isinstance(ct, Izhikevich2007Cell):
        return _IZH
    if isinstance(ct, IafCell):
        return _IAF
    if isinstance(ct, AdExCell):
        return _ADEX
    return None


@dataclass
class SetCell:
    """One `set cell` statement: `values` (field units) for the listed
    instances of `pop` (`ids` None: all, in instance order)."""
    pop: str
    ids: Optional[List[int]]
    prop: str
    values: List[float]


@dataclass
class SetInput:
    """One `set input` statement: `values` (field units) of `prop` for the
    inputs of list `lst` with the given input ids (None: all, by id)."""
    lst: str
    ids: Optional[List[int]]
    prop: str
    values: List[float]


@dataclass
class SetSynapse:
    """One `set synapse` statement: `values` (field units) of the synapse
    type field `prop` for the connections of NeuroML projection `proj` with
    the given connection ids (None: all, by id)."""
    proj: str
    ids: Optional[List[int]]
    prop: str
    values: List[float]


def _synapse_table(st):
    """Settable parameters of a synapse type: NeuroML name -> (field, dimension, factor)."""
    if st.form:
        t = {"tau_syn": ("tau_decay", None, 1.0)}
        if st.form.endswith("CondSynapse"):
            t["e_rev"] = ("erev", None, 1.0)
        return t
    if st.kind == SYN_EXPTHREE:
        return {"gbase1": ("gbase", "conductance", 1.0), "gbase2": ("gbase2", "conductance", 1.0),
                "erev": ("erev", "voltage", 1.0), "tauRise": ("tau_rise", "time", 1.0),
                "tauDecay1": ("tau_decay", "time", 1.0), "tauDecay2": ("tau_decay2", "time", 1.0)}
    if st.kind == SYN_ALPHA_CURRENT:
        return {"tau": ("tau_decay", "time", 1.0), "ibase": ("gbase", "current", 1.0)}
    t = {"gbase": ("gbase", "conductance", 1.0), "erev": ("erev", "voltage", 1.0)}
    if st.kind == SYN_ALPHA:
        t["tau"] = ("tau_decay", "time", 1.0)
    else:
        t["tauDecay"] = ("tau_decay", "time", 1.0)
    if st.kind == SYN_EXPTWO:
        t["tauRise"] = ("tau_rise", "time", 1.0)
    return t


def _proj_members(spec, proj):
    """[(connection id, (projection index, item index))] of NeuroML
    projection `proj`, by connection id."""
    members = []
    for k, pr in enumerate(spec.projections):
        for i, (pid, cid) in enumerate(pr.conn_ids or ()):
            if pid == proj:
                members.append((cid, (k, i)))
    return sorted(members)


def _input_table(obj):
    """Settable properties of an input object: NeuroML name -> (field, dimension, column)."""
    from .network import ClampInputs, PulseInputs
    cur = None if getattr(obj, "dimensionless", False) else "current"
    common = {"delay": ("delay", "time", None), "duration": ("duration", "time", None)}
    if isinstance(obj, PulseInputs):
        return dict(common, amplitude=("amplitude", cur, None))
    if isinstance(obj, ClampInputs):
        t = dict(common, simpleSeriesResistance=("resistance", "resistance", None))
        if obj.triple:
            t.update(conditioningVoltage=("v_before", "voltage", None), testingVoltage=("v_during", "voltage", None),
                     returnVoltage=("v_after", "voltage", None))
        else:
            t.update(targetVoltage=("v_during", "voltage", None))
        return t
    if obj.shape == WAVE_SINE:
        return dict(common, amplitude=("p0", cur, None), period=("p1", "time", None), phase=("p2", None, None))
    return dict(common, startAmplitude=("p0", cur, None), finishAmplitude=("p1", cur, None),
                baselineAmplitude=("p2", cur, None))


def _list_members(spec, lst):
    """(input object, [(input id, item index)]) of inputList `lst`."""
    for obj in list(spec.pulses) + list(spec.waves) + list(spec.clamps):
        if not obj.list_ids:
            continue
        members = [(iid, i) for i, (name, iid) in enumerate(obj.list_ids) if name == lst]
        if members:
            return obj, sorted(members)
    return None, []


def parse(text: str, spec) -> list:
    """The statements of a custom setup file, checked against `spec`."""
    lines = [ln.split("#", 1)[0].split() for ln in text.splitlines()]
    out = []
    i = 0
    while i < len(lines):
        tok = lines[i]
        i += 1
        if not tok:
            continue
        if tok[0] != "set":
            raise ValueError(f"custom setup line {i}: unknown statement {tok[0]!r}")
        if len(tok) >= 2 and tok[1] == "input":
            if len(tok) < 6:
                raise ValueError(f"custom setup line {i}: 'set input' needs list, inputs, property and value")
            lst, ids_s, prop, value = tok[2], tok[3], tok[4], tok[5]
            obj, members = _list_members(spec, lst)
            if obj is None:
                raise ValueError(f"custom setup line {i}: input list {lst} not found (or of a kind 'set input' "
                                 f"does not cover)")
            table = _input_table(obj)
            if prop not in table:
                raise ValueError(f"custom setup line {i}: input list {lst} has no settable property {prop!r}")
            known = [iid for iid, _ in members]
            ids = None
            if ids_s != "all":
                ids = [int(x) for x in ids_s.split(",")]
                if len(set(ids)) != len(ids):
                    raise ValueError(f"custom setup line {i}: an input is listed twice")
                if any(x not in known for x in ids):
                    raise ValueError(f"custom setup line {i}: input not in list {lst}")
            field, dim, _ = table[prop]
            vals, i = _values(lines, i, value, tok[6] if len(tok) > 6 else None, dim, 1.0,
                              len(known) if ids is None else len(ids))
            out.append(SetInput(lst, ids, field, vals))
            continue
        if len(tok) >= 2 and tok[1] == "synapse":
            if len(tok) < 7:
                raise ValueError(f"custom setup line {i}: 'set synapse' needs projection, connections, location, "
                                 f"property and value")
            proj, ids_s, loc, prop, value = tok[2], tok[3], tok[4], tok[5], tok[6]
            members = _proj_members(spec, proj)
            if not members:
                raise ValueError(f"custom setup line {i}: projection {proj} not found (or without connections)")
            if loc != "post":
                raise ValueError(f"custom setup line {i}: location {loc!r}: a spiking connection has its synaptic "
                                 f"component on the 'post' side only")
            known = [cid for cid, _ in members]
            ids = None
            if ids_s != "all":
                ids = [int(x) for x in ids_s.split(",")]
                if len(set(ids)) != len(ids):
                    raise ValueError(f"custom setup line {i}: a connection is listed twice")
                if any(x not in known for x in ids):
                    raise ValueError(f"custom setup line {i}: connection not in projection {proj}")
            k0, _ = members[0][1]
            st = spec.synapse(spec.projections[k0].synapse)
            table = _synapse_table(st)
            if prop not in table:
                raise ValueError(f"custom setup line {i}: synapse {st.name} has no settable property {prop!r}")
            field, dim, factor = table[prop]
            vals, i = _values(lines, i, value, tok[7] if len(tok) > 7 else None, dim, factor,
                              len(known) if ids is None else len(ids))
            out.append(SetSynapse(proj, ids, field, vals))
            continue
        if len(tok) < 2 or tok[1] != "cell":
            raise ValueError(f"custom setup line {i}: 'set {tok[1] if len(tok) > 1 else ''}' is not supported "
                             f"(only 'set cell' on point neurons, 'set input' and 'set synapse')")
        if len(tok) < 7:
            raise ValueError(f"custom setup line {i}: 'set cell' needs population, instances, segments, "
                             f"property and value")
        pop, ids_s, segs, prop, value = tok[2], tok[3], tok[4], tok[5], tok[6]
        pops = {p.name: p for p in spec.populations}
        if pop not in pops:
            raise ValueError(f"custom setup line {i}: population {pop} not found")
        ct = spec.cell_type(pops[pop].cell_type)
        table = _params_of(ct)
        if table is None:
            raise ValueError(f"custom setup line {i}: properties of {type(ct).__name__} cells are not supported "
                             f"(point neurons only)")
        if segs != "all":
            raise ValueError(f"custom setup line {i}: segment specifier must be 'all' for point neurons")
        if prop not in table:
            raise ValueError(f"custom setup line {i}: {type(ct).__name__} has no settable property {prop!r}")
        ids = None
        if ids_s != "all":
            ids = [int(x) for x in ids_s.split(",")]
            if len(set(ids)) != len(ids):
                raise ValueError(f"custom setup line {i}: an instance is listed twice")
            bad = [x for x in ids if not 0 <= x < pops[pop].size]
            if bad:
                raise ValueError(f"custom setup line {i}: instance {bad[0]} not in population {pop}")
        field, dim, factor = table[prop]
        vals, i = _values(lines, i, value, tok[7] if len(tok) > 7 else None, dim, factor,
                          pops[pop].size if ids is None else len(ids))
        out.append(SetCell(pop, ids, field, vals))
    return out


def _values(lines, i, value, unit, dim, factor, n_sel):
    """The statement's values in field units, and the next line index."""
    from .neuroml_io import _UNITS
    scale = 1.0
    if dim is not None:
        if unit is None:
            raise ValueError(f"custom setup line {i}: the property needs units")
        if unit not in _UNITS[dim]:
            raise ValueError(f"custom setup line {i}: unit {unit!r} not known for {dim}")
        scale = _UNITS[dim][unit] * factor
    if value == "multi":
        if i >= len(lines) or not lines[i] or lines[i][0] != "values":
            raise ValueError(f"custom setup line {i}: 'multi' needs a 'values' line after it")
        vals = [float(x) * scale for x in lines[i][1:]]
        i += 1
        if len(vals) != n_sel:
            raise ValueError(f"custom setup line {i}: {len(vals)} values for {n_sel} instances")
    else:
        vals = [float(value) * scale] * n_sel
    return vals, i


def apply_inputs(spec):
    """A copy of `spec` whose input objects carry the `set input`
    statements' values (later statements win); `spec` itself is unchanged."""
    stmts = [st for st in spec.custom_setup if isinstance(st, SetInput)]
    if not stmts:
        return spec
    out = copy.copy(spec)
    out.pulses = [copy.copy(x) for x in spec.pulses]
    out.waves = [copy.copy(x) for x in spec.waves]
    out.clamps = [copy.copy(x) for x in spec.clamps]
    for st in stmts:
        obj, members = _list_members(out, st.lst)
        by_id = dict(members)
        ids = [iid for iid, _ in members] if st.ids is None else st.ids
        arr = np.array(getattr(obj, st.prop), dtype=np.float64, copy=True)
        for iid, v in zip(ids, st.values):
            arr[by_id[iid]] = v
        setattr(obj, st.prop, arr)
    return out


MAX_SYN_TYPES = 32   # synapse types per model the GPU library takes (eden_math.cuh kMaxSynTypes)


def apply_synapses(spec):
    """A copy of `spec` in which the connections that `set synapse`
    statements name use synapse types of their own: one per (synapse type,
    distinct set of overridden values), named `<type>:<n>`, with the
    projections split accordingly (each part keeps its connections' order);
    `spec` itself is unchanged."""
    import dataclasses
    stmts = [st for st in spec.custom_setup if isinstance(st, SetSynapse)]
    if not stmts:
        return spec
    over = {}
    for st in stmts:
        members = _proj_members(spec, st.proj)
        by_id = dict(members)
        ids = [cid for cid, _ in members] if st.ids is None else st.ids
        for cid, v in zip(ids, st.values):
            over.setdefault(by_id[cid], {})[st.prop] = float(v)
    out = copy.copy(spec)
    out.synapses = list(spec.synapses)
    out.projections = []
    derived = {}
    for k, pr in enumerate(spec.projections):
        keys = [tuple(sorted(over.get((k, i), {}).items())) for i in range(len(pr.pre_cell))]
        parts = {}
        for i, key in enumerate(keys):
            parts.setdefault(key, []).append(i)
        for key, idx in parts.items():
            syn = pr.synapse
            if key:
                if (syn, key) not in derived:
                    derived[(syn, key)] = f"{syn}:{len(derived)}"
                    out.synapses.append(dataclasses.replace(spec.synapse(syn), name=derived[(syn, key)], **dict(key)))
                syn = derived[(syn, key)]
            sel = np.array(idx, np.int64)
            out.projections.append(dataclasses.replace(
                pr, name=pr.name if not key else f"{pr.name}:{syn}", synapse=syn, pre_cell=pr.pre_cell[sel],
                post_cell=pr.post_cell[sel], post_seg=pr.post_seg[sel], weight=pr.weight[sel], delay=pr.delay[sel],
                conn_ids=[pr.conn_ids[i] for i in idx] if pr.conn_ids else None))
    if len(out.synapses) > MAX_SYN_TYPES:
        raise ValueError(f"set synapse: {len(out.synapses)} synapse types after the statements, more than the "
                         f"{MAX_SYN_TYPES} a model may have (each distinct set of values is a type)")
    return out


def overrides(spec) -> dict:
    """(population, instance) -> {field: value} after every statement of
    `spec.custom_setup`, later statements overriding earlier ones."""
    res = {}
    pops = {p.name: p for p in spec.populations}
    for st in spec.custom_setup:
        if not isinstance(st, SetCell):
            continue
        ids = list(range(pops[st.pop].size)) if st.ids is None else st.ids
        for inst, v in zip(ids, st.values):
            res.setdefault((st.pop, inst), {})[st.prop] = float(v)
    return res


def write(spec, path: str) -> None:
    """Write `spec.custom_setup` as a setup file (values in field units)."""
    from .neuroml_io import _f
    unit_of = {"voltage": "mV", "capacitance": "pF", "cond_per_voltage": "nS_per_mV", "rate_per_ms": "per_ms",
               "conductance": "nS", "current": "nA", "time": "ms"}
    with open(path, "w") as f:
        for st in spec.custom_setup:
            if isinstance(st, SetInput):
                obj, members = _list_members(spec, st.lst)
                prop, (field, dim, _) = next((k, v) for k, v in _input_table(obj).items() if v[0] == st.prop)
                ids = "all" if st.ids is None else ",".join(str(x) for x in st.ids)
                unit = {None: "", "current": " nA", "time": " ms", "voltage": " mV", "resistance": " Mohm"}[dim]
                f.write(f"set input {st.lst} {ids} {prop} multi{unit}\n")
                f.write("values " + " ".join(_f(v) for v in st.values) + "\n")
                continue
            if isinstance(st, SetSynapse):
                members = _proj_members(spec, st.proj)
                syn = spec.synapse(spec.projections[members[0][1][0]].synapse)
                prop, (field, dim, factor) = next((k, v) for k, v in _synapse_table(syn).items() if v[0] == st.prop)
                ids = "all" if st.ids is None else ",".join(str(x) for x in st.ids)
                f.write(f"set synapse {st.proj} {ids} post {prop} multi" + (f" {unit_of[dim]}" if dim else "") + "\n")
                f.write("values " + " ".join(_f(v / factor) for v in st.values) + "\n")
                continue
            ct = spec.cell_type({p.name: p for p in spec.populations}[st.pop].cell_type)
            prop, (field, dim, factor) = next((k, v) for k, v in _params_of(ct).items() if v[0] == st.prop)
            ids = "all" if st.ids is None else ",".join(str(x) for x in st.ids)
            vals = [v / factor for v in st.values]
            f.write(f"set cell {st.pop} {ids} all {prop} multi {unit_of[dim]}\n")
            f.write("values " + " ".join(_f(v) for v in vals) + "\n")


def apply_to(ct, fields: dict):
    """A copy of cell type `ct` with `fields` overridden."""
    import dataclasses
    return dataclasses.replace(ct, **fields)


__all__ = ["SetCell", "SetInput", "SetSynapse", "parse", "overrides", "write", "apply_to", "apply_inputs",
           "apply_synapses"]
