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
