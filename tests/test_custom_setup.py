"""EdenCustomSetup `set cell` statements on point neurons (host side; the
GPU path runs the lowered per-instance parameters and is checked by the
parity tests over the custom_setup case)."""
import collections

import numpy as np
import pytest

import eden_port
from eden_gb300 import custom_setup, lowering, neuroml_io, workloads
from golden.cases import spec_of
from golden_io import load


def test_overrides_reach_the_lowered_parameters():
    spec = spec_of("custom_setup")
    low = lowering.lower(spec)
    p = low.izh_params
    # izhikevich v0 (index 1) of instances 1 and 3: the last statement on 3 wins
    assert p[1, 1] == np.float32(-64.0) and p[3, 1] == np.float32(-58.0) and p[0, 1] == np.float32(-60.0)
    # the other statements change parameters too
    base = lowering.lower(_without_setup(spec))
    assert (base.izh_params != low.izh_params).any(axis=1).sum() >= 12


def _without_setup(spec):
    import copy
    s = copy.copy(spec)
    s.custom_setup = []
    return s


def test_oracle_needs_the_overrides():
    """A planted mistake in the oracle's input: without the setup file's
    overrides the reference fixture no longer matches."""
    spec = spec_of("custom_setup")
    low = lowering.lower(spec)
    ref, ref_src, _ = load("custom_setup", low)
    assert np.abs(eden_port.run(low)["trace"] - ref).max() < 0.05
    bad = eden_port.run(lowering.lower(_without_setup(spec)))
    assert np.abs(bad["trace"] - ref).max() > 5.0


def test_round_trip(tmp_path):
    spec = spec_of("custom_setup")
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    np.testing.assert_array_equal(lowering.lower(spec).izh_params, lowering.lower(back).izh_params)


@pytest.mark.parametrize("text,match", [
    ("set input Input0 0 amplitude 14\n", "not found"),
    ("set input stim_izh 0 period 2 ms\n", "settable"),
    ("set input stim_izh 9 amplitude 0.1 nA\n", "not in list"),
    ("set synapse proj all post erev 0.05 V\n", "not found"),
    ("set dendrite proj all post erev 0.05 V\n", "not supported"),
    ("set cell izh 1 all v0 -64\n", "units"),
    ("set cell izh 1 all w0 -64 mV\n", "settable"),
    ("set cell izh 1,1 all v0 -64 mV\n", "twice"),
    ("set cell izh 9 all v0 -64 mV\n", "not in population"),
    ("set cell izh all all d multi pA\nvalues 1 2\n", "values for"),
    ("set cell izh 1 soma v0 -64 mV\n", "segment"),
])
def test_unsupported_or_malformed_statements_are_refused(text, match):
    with pytest.raises(ValueError, match=match):
        custom_setup.parse(text, spec_of("custom_setup"))


def test_physical_cells_are_refused():
    spec = workloads.single_comp_hh(n_cells=2, length_ms=1.0)
    with pytest.raises(ValueError, match="point neurons only"):
        custom_setup.parse(f"set cell {spec.populations[0].name} all all v -60 mV\n", spec)


def test_oracle_needs_the_input_statements():
    """Dropping only the 'set input' statements: the fixture no longer matches."""
    import copy
    spec = spec_of("custom_setup")
    ref, _, _ = load("custom_setup", lowering.lower(spec))
    s = copy.copy(spec)
    s.custom_setup = [st for st in spec.custom_setup if not isinstance(st, custom_setup.SetInput)]
    assert len(s.custom_setup) < len(spec.custom_setup)
    bad = eden_port.run(lowering.lower(s))
    assert np.abs(bad["trace"] - ref).max() > 5.0


def _read_back(spec, tmp_path):
    """`spec` written as NeuroML and read again: its connections then carry
    the (projection id, connection id) that `set synapse` names."""
    return neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))


def test_synapse_statements_give_connections_types_of_their_own(tmp_path):
    spec = _read_back(spec_of("alpha_synapses"), tmp_path / "a")
    # the writer makes a projection per run of one (pre, post) population
    # pair; these three hold 4, 3 and 5 connections
    size = collections.Counter(pid for pr in spec.projections for pid, _ in pr.conn_ids)
    assert (size["proj_syn_e2_4"], size["proj_syn_alpha_i_16"], size["proj_syn_alpha_10"]) == (4, 3, 5)
    spec.custom_setup = custom_setup.parse(
        "set synapse proj_syn_e2_4 all post erev 0.01 V\n"
        "set synapse proj_syn_e2_4 1,3 post tauRise multi msec\nvalues 0.25 0.5\n"
        "set synapse proj_syn_alpha_i_16 0 post ibase 20 pA\n"
        "set synapse proj_syn_alpha_10 2 post tau 0.004 sec\n", spec)
    base = lowering.lower(_without_setup(spec))
    low = lowering.lower(spec)
    n0 = len(base.syn_types)
    # e2: one type for connections 1 and 3 each (their tauRise differs) and
    # one for the other two (erev only); one alphaCurrent and one alpha type
    assert len(low.syn_types) == n0 + 5
    types = custom_setup.apply_synapses(spec).synapses
    of = lambda prefix: [st for st in types if st.name.startswith(prefix)]
    e2 = spec.synapse("syn_e2")
    assert [st.erev for st in of("syn_e2:")] == [10.0] * 3
    assert sorted(st.tau_rise for st in of("syn_e2:")) == sorted([e2.tau_rise, 0.25, 0.5])
    assert [(st.gbase, st.kind) for st in of("syn_alpha_i:")] == [(0.02, spec.synapse("syn_alpha_i").kind)]
    assert [st.tau_decay for st in of("syn_alpha:")] == [4.0]
    # every connection keeps its target; only the 6 named ones change type
    assert sorted(zip(low.syn_target.tolist(), low.syn_weight.tolist())) == \
        sorted(zip(base.syn_target.tolist(), base.syn_weight.tolist()))
    assert (low.syn_type >= n0).sum() == 4 + 1 + 1
    # and the oracle sees the difference
    assert np.abs(eden_port.run(low)["trace"] - eden_port.run(base)["trace"]).max() > 0.1
    # round trip: the setup file names the same projections and connections
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path / "b")))
    low2 = lowering.lower(back)
    np.testing.assert_array_equal(low2.syn_types, low.syn_types)
    np.testing.assert_array_equal(low2.syn_type, low.syn_type)
    np.testing.assert_array_equal(low2.syn_target, low.syn_target)


@pytest.mark.parametrize("text,match", [
    ("set synapse proj_syn_e2_4 all pre erev 0 mV\n", "post"),
    ("set synapse proj_syn_e2_4 all post tau 2 ms\n", "settable"),
    ("set synapse proj_syn_alpha_10 all post tauDecay 2 ms\n", "settable"),
    ("set synapse proj_syn_e2_4 99 post erev 0 mV\n", "not in projection"),
    ("set synapse proj_syn_e2_4 1,1 post erev 0 mV\n", "twice"),
    ("set synapse proj_syn_e2_4 all post erev 0\n", "units"),
    ("set synapse proj_syn_e2_4 1,2 post erev multi mV\nvalues 1\n", "values for"),
    ("set synapse proj_syn_e2_4 all post erev\n", "needs"),
])
def test_malformed_synapse_statements_are_refused(text, match, tmp_path):
    spec = _read_back(spec_of("alpha_synapses"), tmp_path)
    with pytest.raises(ValueError, match=match):
        custom_setup.parse(text, spec)


def test_too_many_distinct_synapse_values_are_refused(tmp_path):
    spec = _read_back(spec_of("izh_net"), tmp_path)
    pid, n = collections.Counter(pid for pr in spec.projections for pid, _ in pr.conn_ids).most_common(1)[0]
    assert n > 40
    spec.custom_setup = custom_setup.parse(
        f"set synapse {pid} all post tauDecay multi ms\nvalues " + " ".join(str(1 + 0.01 * k) for k in range(n)) + "\n",
        spec)
    with pytest.raises(ValueError, match="more than the 32"):
        lowering.lower(spec)
