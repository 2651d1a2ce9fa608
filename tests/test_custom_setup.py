"""EdenCustomSetup `set cell` statements on point neurons (host side; the
GPU path runs the lowered per-instance parameters and is checked by the
parity tests over the custom_setup case)."""
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
    ("set synapse proj all post erev 0.05 V\n", "not supported"),
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
