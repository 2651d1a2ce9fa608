"""LEMS/NeuroML front end: writing a seeded network and reading it back gives
the same lowered model, field for field (the reader is what `eden nml` and
runEden() use on user files)."""
import numpy as np
import pytest

from eden_gb300 import lowering, neuroml_io, workloads
from golden.cases import spec_of


def _same(a, b):
    bad = []
    for f in a.__dataclass_fields__:
        x, y = getattr(a, f), getattr(b, f)
        if isinstance(x, np.ndarray):
            if x.dtype.names:
                ok = all(np.array_equal(x[n], y[n], equal_nan=True) for n in x.dtype.names)
            else:
                ok = x.shape == y.shape and np.array_equal(x, y, equal_nan=x.dtype.kind == "f")
        else:
            ok = x == y
        if not ok:
            bad.append(f)
    return bad


@pytest.mark.parametrize("name,kw", [
    ("single_comp_hh", dict(n_cells=8, length_ms=5.0)),
    ("multicomp_net", dict(n_cells=6, in_degree=4, length_ms=5.0, max_seg=30)),
    ("izh_net", dict(n_cells=20, in_degree=5, length_ms=5.0)),
    ("ball_and_stick", dict(n_inst=3, length_ms=5.0)),
    ("gap_junctions", dict(length_ms=5.0)),
    ("alpha_synapses", dict(length_ms=5.0)),
])
def test_write_read_round_trip(tmp_path, name, kw):
    spec = workloads.CONFIGS[name](**kw)
    path = neuroml_io.write_lems(spec, str(tmp_path))
    back = neuroml_io.read_lems(path)
    assert _same(lowering.lower(spec), lowering.lower(back)) == []


def test_unsupported_elements_fail_loudly(tmp_path):
    spec = workloads.single_comp_hh(n_cells=2, length_ms=1.0)
    path = neuroml_io.write_lems(spec, str(tmp_path))
    nml = tmp_path / f"{spec.name}.nml"
    text = nml.read_text().replace("<pulseGenerator ", "<pulseGeneratorDL ")
    nml.write_text(text.replace("</pulseGenerator>", "</pulseGeneratorDL>"))
    with pytest.raises(ValueError):
        neuroml_io.read_lems(path)


def test_units_follow_reference_scales(tmp_path):
    spec = workloads.single_comp_hh(n_cells=1, length_ms=1.0)
    path = neuroml_io.write_lems(spec, str(tmp_path))
    nml = tmp_path / f"{spec.name}.nml"
    text = nml.read_text().replace('condDensity="120.0 mS_per_cm2"', 'condDensity="1200.0 S_per_m2"')
    text = text.replace('erev="50.0mV"', 'erev="0.05V"')
    nml.write_text(text)
    a = lowering.lower(spec)
    b = lowering.lower(neuroml_io.read_lems(path))
    np.testing.assert_allclose(a.chan_gbase, b.chan_gbase, rtol=1e-7)
    np.testing.assert_allclose(a.chan_erev, b.chan_erev, rtol=1e-7)


def test_electrical_connection_forms(tmp_path):
    """electricalConnection (cell indices, weight 1) and conductances in pS
    read as the weighted instance form with nS does."""
    spec = workloads.gap_junctions(length_ms=5.0)
    path = neuroml_io.write_lems(spec, str(tmp_path))
    nml = tmp_path / f"{spec.name}.nml"
    text = nml.read_text().replace('conductance="4.0nS"', 'conductance="4000.0pS"')
    nml.write_text(text)
    a = lowering.lower(spec)
    b = lowering.lower(neuroml_io.read_lems(path))
    assert _same(a, b) == []
    # the index form: preCell="i", no weight
    import re
    text = re.sub(r'<electricalConnectionInstanceW id="(\d+)" preCell="\.\./\w+/(\d+)/\w+" preSegment="(\d+)" '
                  r'postCell="\.\./\w+/(\d+)/\w+" postSegment="(\d+)" synapse="(\w+)" weight="[^"]*"/>',
                  r'<electricalConnection id="\1" preCell="\2" preSegment="\3" postCell="\4" postSegment="\5" '
                  r'synapse="\6"/>', text)
    assert "electricalConnectionInstanceW" not in text
    nml.write_text(text)
    c = lowering.lower(neuroml_io.read_lems(path))
    np.testing.assert_array_equal(c.gap_target, a.gap_target)
    np.testing.assert_array_equal(c.gap_peer, a.gap_peer)
    np.testing.assert_array_equal(c.gap_conductance, a.gap_conductance)
    np.testing.assert_array_equal(c.gap_weight, np.ones_like(a.gap_weight))


def test_gap_junctions_on_point_neurons_fail_loudly():
    from eden_gb300.network import ElectricalProjection
    spec = workloads.gap_junctions(length_ms=5.0)
    iz = spec.populations[0].size + spec.populations[1].size
    spec.electrical.append(ElectricalProjection("bad", "gap_weak", np.array([0]), np.array([0]), np.array([iz]),
                                                np.array([0]), np.array([1.0])))
    with pytest.raises(ValueError, match="physical cells"):
        lowering.lower(spec)


def test_pynn_and_exp_three_synapses_round_trip(tmp_path):
    """expCondSynapse, alphaCondSynapse, expCurrSynapse, alphaCurrSynapse and
    expThreeSynapse are written back as themselves and lower to the same
    tables; an expThreeSynapse lowers to two expTwo types on every one of
    its connections and timed inputs."""
    spec = spec_of("pynn_synapses")
    low = lowering.lower(spec)
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    assert [(s.kind, s.form) for s in back.synapses] == [(s.kind, s.form) for s in spec.synapses]
    low2 = lowering.lower(back)
    np.testing.assert_array_equal(low2.syn_types, low.syn_types)
    np.testing.assert_array_equal(low2.syn_target, low.syn_target)
    np.testing.assert_array_equal(low2.syn_type, low.syn_type)
    n3 = len(next(p for p in spec.projections if p.synapse == "syn_e3").pre_cell)
    n_conn = sum(len(p.pre_cell) for p in spec.projections)
    assert len(low.syn_target) == n_conn + n3
    # a Poisson input draws one train: it cannot drive an expThreeSynapse's two parts
    import copy
    bad = copy.deepcopy(spec)
    bad.poissons[0].synapse = "syn_e3"
    with pytest.raises(ValueError, match="expThreeSynapse"):
        lowering.lower(bad)


def test_continuous_projections_round_trip(tmp_path):
    """continuousConnectionInstanceW with linearGraded, graded, silent and
    gapJunction components on either end, and a linearGradedSynapse on an
    electrical connection: written and read back to the same lowered ends."""
    spec = spec_of("continuous_synapses")
    low = lowering.lower(spec)
    assert len(low.graded_target) == 2 + 2 * 2 + 2 and len(low.gap_target) == 2 + 2 + 2 + 2 * 2
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    assert [(g.name, g.kind) for g in back.gap_types] == [(g.name, g.kind) for g in spec.gap_types]
    low2 = lowering.lower(back)
    for f in ("gap_target", "gap_peer", "gap_conductance", "gap_weight", "graded_target", "graded_peer",
              "graded_params", "graded_weight"):
        np.testing.assert_array_equal(getattr(low2, f), getattr(low, f), err_msg=f)


def test_blocking_plastic_synapse_round_trip(tmp_path):
    """The reference's CoreSynapses network (every core synapse): the
    blockingPlasticSynapse keeps its block and plasticity mechanisms through
    a write and a read, and the lowered tables are the same."""
    import reference_runner
    path = reference_runner.validation_network("LEMS_EdenTest_CoreSynapses.xml")
    if path is None:
        pytest.skip("reference tree not present")
    spec = neuroml_io.read_lems(path)
    bp = next(s for s in spec.synapses if s.block)
    assert bp.plasticity["type"] == "tsodyksMarkramDepFacMechanism" and bp.block["scalingVolt"] == 150.0
    low = lowering.lower(spec)
    back = neuroml_io.read_lems(neuroml_io.write_lems(spec, str(tmp_path)))
    low2 = lowering.lower(back)
    np.testing.assert_array_equal(low2.syn_types, low.syn_types)
    for f in ("syn_target", "syn_type", "gap_target", "gap_peer", "graded_target", "graded_params"):
        np.testing.assert_array_equal(getattr(low2, f), getattr(low, f), err_msg=f)
    # connections only: a Poisson input on it is refused
    import copy
    bad = copy.deepcopy(spec)
    from eden_gb300.network import PoissonInputs
    bad.poissons.append(PoissonInputs("*", bp.name, 10.0, np.array([1]), np.array([0])))
    with pytest.raises(ValueError, match="connections only"):
        lowering.lower(bad)
