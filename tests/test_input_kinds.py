"""sineGenerator / rampGenerator inputs and the numbering of Poisson inputs'
random draws (host side and oracle; the GPU path is checked against both by
the parity tests over the input_kinds case).

The reference numbers a cell type's random() calls compartment by
compartment and, within a compartment, Poisson component by Poisson
component in definition order (eden/Eden.cpp:1812-1830, 2450-2458, 5943,
6540); the draws of a Poisson input use that number and the next."""
import numpy as np
import pytest

import eden_port
from eden_gb300 import lowering, neuroml_io, workloads
from eden_gb300.network import (WAVE_RAMP, WAVE_SINE, NetworkSpec, PhysicalCell, PoissonInputs, Population,
                                SynapseType, SYN_EXPTWO, WaveInputs, hh_channels)
from golden.cases import spec_of
from golden_io import load


def _two_pop_spec():
    spec = NetworkSpec("rng", 0.025, 5.0, 7, channels=hh_channels())
    spec.synapses.append(SynapseType("s", SYN_EXPTWO, gbase=1.0, erev=0.0, tau_decay=5.0, tau_rise=0.5))
    parent = np.array([-1, 0, 1, 0])
    dens = workloads._hh_densities(4, np.array([True, False, False, False]))
    spec.cells.append(PhysicalCell("c", parent, np.full(4, 20.0), np.full(4, 2.0), dens, 1.0, 150.0, -65.0, -20.0))
    spec.populations.append(Population("a", "c", 2))
    spec.populations.append(Population("b", "c", 1))
    # component 0 on soma of cell 0 only; component 1 on soma of cell 2 and
    # compartment 2 of cell 1; component 2 on compartment 3 of cell 0
    spec.poissons.append(PoissonInputs("*", "s", 10.0, np.array([0, 0]), np.array([0, 0])))
    spec.poissons.append(PoissonInputs("*", "s", 10.0, np.array([2, 1]), np.array([0, 2])))
    spec.poissons.append(PoissonInputs("*", "s", 10.0, np.array([0]), np.array([3])))
    return spec


def test_rng_bases_follow_compartments_and_component_order():
    low = lowering.lower(_two_pop_spec())
    base = {(int(t), int(b)) for t, b in zip(low.pois_target, low.pois_rng_base)}
    # the cell type's compartment 0 carries components {0, 1} (union over the
    # type's cells, whichever population): draws 0-1 and 2-3; compartment 2
    # carries {1} after compartment 0's four calls: 4-5; compartment 3
    # carries {2} after six: 6-7
    cell0, cell1, cell2 = 0, 4, 8
    assert base == {(cell0, 0), (cell2, 2), (cell1 + 2, 4), (cell0 + 3, 6)}


def test_rng_bases_of_the_input_kinds_case():
    spec = spec_of("input_kinds")
    low = lowering.lower(spec)
    soma_targets = set(low.gid_target_base[:6].tolist())
    by_target = {}
    for t, b in zip(low.pois_target, low.pois_rng_base):
        by_target.setdefault(int(t), set()).add(int(b))
    # three components can meet on a soma (ids 0, 2, 4); dendrite 2 follows
    # the soma's six calls, dendrite 4 those and dendrite 2's two
    assert all(by_target[t] <= {0, 2, 4} for t in soma_targets)
    assert by_target[int(low.gid_target_base[1]) + 2] == {6}
    assert by_target[int(low.gid_target_base[0]) + 4] == {8}
    iz = int(low.gid_target_base[6])
    assert by_target[iz] == {0, 2}


def test_oracle_needs_the_rng_numbering():
    """A planted mistake in the oracle: with every input's draws numbered from
    0, as for a lone Poisson component, the reference fixture no longer
    matches."""
    low = lowering.lower(spec_of("input_kinds"))
    ref, _, _ = load("input_kinds", low)
    good = eden_port.run(low)
    assert np.abs(good["trace"] - ref).max() < 0.05
    low.pois_rng_base = None
    bad = eden_port.run(low)
    assert np.abs(bad["trace"] - ref).max() > 5.0


def _wave_spec(shape, p0, p1, p2, delay=2.0, duration=5.0, weight=1.5):
    spec = NetworkSpec("wave", 0.025, 10.0, 1, channels=hh_channels())
    dens = workloads._hh_densities(1, np.zeros(1, bool))
    spec.cells.append(PhysicalCell("p", np.array([-1]), np.array([0.0]), np.array([20.0]), dens, 1.0, 150.0,
                                   -65.0, -20.0))
    spec.populations.append(Population("p", "p", 1))
    one = lambda x: np.array([x], dtype=float)
    spec.waves.append(WaveInputs(shape, np.array([0]), np.array([0]), one(delay), one(duration), one(p0), one(p1),
                                 one(p2), one(weight)))
    from eden_gb300.network import OutputColumn
    spec.trace_columns = [OutputColumn("p", 0, 0)]
    return spec


def _injected_current(spec):
    """The current (nA) the oracle's passive compartment received at each
    step, recovered from its trace: C dV/dt = I - g (V - E) in the
    backward-Euler form the loop uses is linear in I, so the difference to
    the run without the input gives it up to the membrane filter."""
    low = lowering.lower(spec)
    with_in = eden_port.run(low)["trace"][:, 0].astype(np.float64)
    spec.waves.clear()
    without = eden_port.run(lowering.lower(spec))["trace"][:, 0].astype(np.float64)
    return with_in - without


def test_sine_is_zero_outside_its_window_and_follows_the_phase():
    dv = _injected_current(_wave_spec(WAVE_SINE, 0.2, 2.0, 0.5))
    t = np.arange(len(dv)) * 0.025
    assert np.all(dv[t < 2.0] == 0.0)
    inside = (t > 2.2) & (t < 6.9)
    assert np.any(dv[inside] > 0) and np.any(dv[inside] < 0)   # a full period swings both ways


def test_ramp_holds_its_baseline_before_the_ramp():
    dv = _injected_current(_wave_spec(WAVE_RAMP, 0.0, 0.3, 0.1))
    t = np.arange(len(dv)) * 0.025
    # the baseline drives the compartment from the first step on
    assert dv[1] > 0 and np.all(np.diff(dv[(t > 0.05) & (t < 2.0)]) > 0)


def test_neuroml_round_trip_keeps_waves_and_poisson_order(tmp_path):
    spec = spec_of("input_kinds")
    lems = neuroml_io.write_lems(spec, str(tmp_path))
    back = neuroml_io.read_lems(lems)
    a, b = lowering.lower(spec), lowering.lower(back)
    for f in ("wave_target", "wave_shape", "wave_params", "wave_weight", "pulse_weight", "pois_target", "pois_rng_base",
              "pois_instance", "pois_rate", "timed_target"):
        np.testing.assert_array_equal(np.asarray(getattr(a, f)), np.asarray(getattr(b, f)), err_msg=f)


def test_transient_poisson_is_refused(tmp_path):
    spec = spec_of("input_kinds")
    lems = neuroml_io.write_lems(spec, str(tmp_path))
    nml = [p for p in tmp_path.iterdir() if p.suffix == ".nml"][0]
    txt = nml.read_text().replace("<poissonFiringSynapse id=\"poisson0\" ",
                                  "<transientPoissonFiringSynapse id=\"poisson0\" delay=\"1ms\" duration=\"2ms\" ")
    nml.write_text(txt)
    with pytest.raises(ValueError, match="transientPoissonFiringSynapse"):
        neuroml_io.read_lems(lems)


def test_unknown_wave_shape_is_refused():
    spec = _wave_spec(WAVE_SINE, 0.2, 2.0, 0.5)
    spec.waves[0].shape = "square"
    with pytest.raises(ValueError, match="shape"):
        lowering.lower(spec)


def test_voltage_clamp_round_trip(tmp_path):
    spec = spec_of("voltage_clamps")
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    a, b = lowering.lower(spec), lowering.lower(back)
    for f in ("clamp_target", "clamp_params", "clamp_weight"):
        np.testing.assert_array_equal(np.asarray(getattr(a, f)), np.asarray(getattr(b, f)), err_msg=f)
    # a voltageClamp has no current before its delay or after delay + duration
    simple = ~np.isnan(a.clamp_params[:, 3]) & np.isnan(a.clamp_params[:, 2])
    assert simple.sum() == 8 and np.isnan(a.clamp_params[simple, 4]).all()


def test_inactive_triple_clamp_is_refused(tmp_path):
    lems = neuroml_io.write_lems(spec_of("voltage_clamps"), str(tmp_path))
    nml = tmp_path / "voltage_clamps.nml"
    nml.write_text(nml.read_text().replace('active="1"', 'active="0"'))
    with pytest.raises(ValueError, match="active"):
        neuroml_io.read_lems(lems)


def test_dimensionless_inputs_round_trip_and_dimension_checks(tmp_path):
    spec = spec_of("dl_inputs")
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    a, b = lowering.lower(spec), lowering.lower(back)
    for f in ("pulse_target", "pulse_amplitude", "pulse_weight", "wave_target", "wave_params", "izh_params",
              "izh_kind"):
        np.testing.assert_array_equal(np.asarray(getattr(a, f)), np.asarray(getattr(b, f)), err_msg=f)
    assert (a.izh_kind == lowering.POINT_IZH_DL).sum() == 6
    # a dimensional pulse into an izhikevichCell, and a DL pulse into an izhikevich2007Cell, are refused
    bad = spec_of("dl_inputs")
    bad.pulses[0].dimensionless = False
    with pytest.raises(ValueError, match="dimensionless"):
        lowering.lower(bad)
    bad = spec_of("dl_inputs")
    bad.pulses[1].dimensionless = True
    with pytest.raises(ValueError, match="dimensionless"):
        lowering.lower(bad)
