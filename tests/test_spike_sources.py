"""Spike sources with no membrane (spikeArray, spikeGenerator): the steps at
which they emit, against the reference's own output on a hand-written case,
their NeuroML round trip, and what they cannot be (a target)."""
import os
import tempfile

import numpy as np
import pytest

from eden_gb300 import lowering, neuroml_io, workloads
from eden_gb300.network import (EventSelection, NetworkSpec, OutputColumn, Population, SpikeArrayCell,
                                SpikeGeneratorCell)


def test_emission_steps_match_the_reference():
    # the reference (oracle/_ref/eden) run on spikeArray times 1, 2.5, 2.51,
    # 7.0125 and 0 ms and a 2.3 ms spikeGenerator at dt 0.025 ms logged
    # spikes at 0.025, 1.025, 2.525, 7.025 ms and 2.325, 4.625, 6.925, 9.225,
    # 11.525 ms: a spike-list time T is emitted in the first step whose
    # t + dt exceeds it (two times in one step give one spike), and the
    # spike is logged at the next step
    src, step = lowering.spike_source_steps(
        {"a": (SpikeArrayCell("a", np.array([1.0, 2.5, 2.51, 7.0125, 0.0])), [0, 1]),
         "g": (SpikeGeneratorCell("g", 2.3), [2])}, np.float32(25.0), 481)
    logged_ms = {s: sorted(((k - 1) * 0.025) for k in step[src == s]) for s in (0, 1, 2)}
    np.testing.assert_allclose(logged_ms[0], [0.025, 1.025, 2.525, 7.025], atol=1e-9)
    np.testing.assert_allclose(logged_ms[1], logged_ms[0])
    np.testing.assert_allclose(logged_ms[2], [2.325, 4.625, 6.925, 9.225, 11.525], atol=1e-9)
    assert np.all(np.diff(step) >= 0)


def test_generator_spikes_stop_at_the_run_length():
    src, step = lowering.spike_source_steps({"g": (SpikeGeneratorCell("g", 1.0), [0])}, np.float32(25.0), 401)
    assert step.max() <= 402 and len(step) == 10


def test_neuroml_round_trip():
    spec = workloads.spike_sources(length_ms=20.0)
    with tempfile.TemporaryDirectory() as d:
        back = neuroml_io.read_lems(neuroml_io.write_lems(spec, d))
    a, b = lowering.lower(spec), lowering.lower(back)
    np.testing.assert_array_equal(a.ext_src, b.ext_src)
    np.testing.assert_array_equal(a.ext_step, b.ext_step)
    np.testing.assert_array_equal(a.syn_src, b.syn_src)
    assert (a.src_target == -1).sum() == sum(p.size for p in spec.populations if p.name.startswith("ps"))


def test_a_spike_source_is_not_a_target():
    spec = NetworkSpec("x", 0.025, 1.0, 1)
    spec.cells.append(SpikeArrayCell("sa", np.array([0.5])))
    spec.populations.append(Population("p", "sa", 1))
    spec.trace_columns = [OutputColumn("p", 0, 0)]
    spec.event_selections = [EventSelection("p", 0, 0)]
    with pytest.raises(ValueError, match="no membrane"):
        lowering.lower(spec)


def test_event_set_steps_match_the_reference(tmp_path):
    # the reference run on this file, with zero-delay expTwo connections
    # from each (instance, port) to its own izhikevich cell, fired the
    # synapses of 0!0 in step 2, of 1!0 in step 42 and of 0!1 and 1!1 in
    # step 82: a frame is applied in the first step whose time less 1e-9 s
    # exceeds its timestamp, and the synapses read it in that step; the
    # frame at 0.0019 s follows a later one and is ignored
    from eden_gb300.network import EventSetReaderCell
    f = tmp_path / "events.txt"
    f.write_text("0.000000 0\n0.001000 1!0\n0.002000 0!1 1!1\n0.0019 1\n0.002512 0!0 0!1\n"
                 "0.0025125 1!1\n0.004000 1!0\n0.004010 0\n")
    frames = neuroml_io.read_event_set(str(f), 2, 2)
    assert len(frames) == 8 and frames[2][1] == [(0, 1), (1, 1)]
    reader = EventSetReaderCell("r", 2, ["zero", "one"], frames)
    src, step = lowering.spike_source_steps({"r": (reader, [10, 11, 12, 13])}, np.float32(25.0), 321)
    got = sorted(zip(src.tolist(), step.tolist()))
    want = sorted([(10, 2), (12, 42), (11, 82), (13, 82), (10, 102), (11, 102), (13, 102), (12, 162), (10, 162)])
    assert got == want


def test_event_set_round_trip():
    spec = workloads.event_sets(length_ms=20.0)
    with tempfile.TemporaryDirectory() as d:
        lems = neuroml_io.write_lems(spec, d)
        assert os.path.exists(os.path.join(d, "evr_events.txt"))
        back = neuroml_io.read_lems(lems)
    a, b = lowering.lower(spec), lowering.lower(back)
    np.testing.assert_array_equal(a.ext_src, b.ext_src)
    np.testing.assert_array_equal(a.ext_step, b.ext_step)
    np.testing.assert_array_equal(a.syn_src, b.syn_src)
    # reader sources follow the cells: the cells' global ids (and RNG seeds) are unchanged
    assert a.event_src.max() < a.ext_src.min()


def test_point_neuron_round_trip_and_kinds():
    from eden_gb300.lowering import (POINT_ADEX, POINT_IAF, POINT_IAF_REF, POINT_IAF_TAU, POINT_IAF_TAU_REF,
                                     POINT_PARAMS)
    spec = workloads.point_neurons(n_per_kind=2, length_ms=5.0)
    with tempfile.TemporaryDirectory() as d:
        back = neuroml_io.read_lems(neuroml_io.write_lems(spec, d))
    a, b = lowering.lower(spec), lowering.lower(back)
    np.testing.assert_array_equal(a.izh_kind, [POINT_IAF_TAU] * 2 + [POINT_IAF_TAU_REF] * 2 + [POINT_IAF] * 2 +
                                  [POINT_IAF_REF] * 2 + [POINT_ADEX] * 2)
    assert a.izh_params.shape == (10, POINT_PARAMS)
    np.testing.assert_array_equal(a.izh_params, b.izh_params)
    # adExIaF in engine units: pF, uS, mV, us, nA
    np.testing.assert_allclose(a.izh_params[-1, :11], [281.0, 0.03, -70.6, -50.4, -40.4, -48.5, 2.0, 40000.0,
                                                       a.izh_params[-1, 8], 0.004, 0.08], rtol=1e-6)


def test_current_into_tau_cells_is_refused():
    spec = workloads.point_neurons(n_per_kind=2, length_ms=5.0)
    spec.pulses[0].cell = spec.pulses[0].cell.copy()
    spec.pulses[0].cell[0] = 0                     # an iafTauCell
    with pytest.raises(ValueError, match="do not receive current"):
        lowering.lower(spec)


def test_timed_input_steps_and_round_trip():
    # the first step whose t + dt exceeds each time, once per step; times
    # before the run fire in step 1, times after it never
    th = (lowering.step_times_f32(np.float32(25.0), 401) + np.float32(25.0)).astype(np.float32)
    steps = lowering.timed_steps([-1.0, 0.0, 0.01, 2.5, 2.51, 2.525, 10.0, 10.01, 50.0], th)
    np.testing.assert_array_equal(steps, [1, 101, 102, 401])
    spec = workloads.timed_inputs(length_ms=20.0)
    with tempfile.TemporaryDirectory() as d:
        back = neuroml_io.read_lems(neuroml_io.write_lems(spec, d))
    a, b = lowering.lower(spec), lowering.lower(back)
    for f in ("timed_target", "timed_type", "timed_weight", "timed_off", "timed_step"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f))
    assert a.timed_step.min() >= 1


def test_random_generators_emit_in_the_reference_steps():
    """spikeGeneratorRandom / Poisson / RefPoisson spikes are computed on the
    host with the reference's hash RNG (the cell's seed, its LEMS code's
    instance, the step, call id 0 for the OnStart draw and 1 after): every
    source's logged steps equal the reference's own output, spike for spike
    (tests/golden/random_sources.npz)."""
    from golden.cases import spec_of
    from golden_io import load
    low = lowering.lower(spec_of("random_sources"))
    _, ref_src, ref_step = load("random_sources", low)
    n_src = 12
    for g in range(n_src):
        mine = np.sort(low.ext_step[low.ext_src == g])
        np.testing.assert_array_equal(mine, np.sort(ref_step[ref_src == g]), err_msg=f"source {g}")
        assert len(mine) >= 5


def test_random_generator_round_trip(tmp_path):
    from golden.cases import spec_of
    spec = spec_of("random_sources")
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    a, b = lowering.lower(spec), lowering.lower(back)
    np.testing.assert_array_equal(a.ext_src, b.ext_src)
    np.testing.assert_array_equal(a.ext_step, b.ext_step)
