"""Seeded networks shared by the golden fixtures and the parity tests.

Each case is (generator name, keyword arguments, box tolerance in mV, time
window compared in ms or None for the whole run).  The recurrent
multicompartment network is chaotic -- single-precision rounding moves a spike
by a step and the difference grows -- so it is compared over its first 15 ms.
"""
CASES = {
    "single_comp_hh": ("single_comp_hh", dict(n_cells=64, length_ms=100.0, n_recorded=6), 1.0, None),
    "izh_net": ("izh_net", dict(n_cells=300, in_degree=20, length_ms=100.0, n_recorded=6), 1.0, None),
    "multicomp_poisson": ("multicomp_net", dict(n_cells=24, in_degree=20, length_ms=60.0, max_seg=80, weight=0.0,
                                                n_recorded=6), 1.0, None),
    "multicomp_recurrent": ("multicomp_net", dict(n_cells=24, in_degree=20, length_ms=15.0, max_seg=80,
                                                  n_recorded=6), 1.0, None),
    "ball_and_stick": ("ball_and_stick", dict(n_inst=8, length_ms=40.0), 1.0, None),
    "spike_sources": ("spike_sources", dict(), 1.0, None),
    "event_sets": ("event_sets", dict(), 1.0, None),
    "point_neurons": ("point_neurons", dict(), 1.0, None),
    "timed_inputs": ("timed_inputs", dict(), 1.0, None),
    "input_kinds": ("input_kinds", dict(), 1.0, None),
    "gate_kinds": ("gate_kinds", dict(), 1.0, None),
    "voltage_clamps": ("voltage_clamps", dict(), 1.0, None),
    "random_sources": ("random_sources", dict(), 1.0, None),
    "custom_setup": ("custom_setup", dict(), 1.0, None),
    "dl_inputs": ("dl_inputs", dict(), 1.0, None),
    "gap_junctions": ("gap_junctions", dict(), 1.0, None),
    "alpha_synapses": ("alpha_synapses", dict(), 1.0, None),
    "pynn_synapses": ("pynn_synapses", dict(), 1.0, None),
    "continuous_synapses": ("continuous_synapses", dict(), 1.0, None),
    # the reference's `cable_solver fwd_euler` (an explicit cable update):
    # HH ball-and-stick cells with five dendrite compartments, and the
    # branched cells of the input-kinds case (stable at dt 0.025 ms, unlike
    # the finer compartments of the other multicompartment cases)
    "ball_and_stick_fwd": ("ball_and_stick", dict(n_inst=8, n_dend=5, length_ms=40.0, cable_solver="fwd_euler"),
                           1.0, None),
    "input_kinds_fwd": ("input_kinds", dict(cable_solver="fwd_euler"), 1.0, None),
}


# The configurations at (or near) their stated sizes, for the full-size GPU
# tests: C1 as stated (1,000 single-compartment HH cells, 1 s, 10 recorded
# cells; its trajectory is stored every `stride`-th sample) and C3 reduced to
# 10,000 cells (in-degree 100, 1 M expOne synapses) over 100 ms.
# name -> (generator, keyword arguments, trajectory stride)
FULL_CASES = {
    "c1_full": ("single_comp_hh", dict(n_cells=1000, length_ms=1000.0, n_recorded=10), 8),
    "c3_10k": ("izh_net", dict(n_cells=10000, in_degree=100, length_ms=100.0, n_recorded=10), 1),
}


def spec_of(name):
    """The case's network; a `cable_solver` entry among its arguments is the
    simulator setting (the reference's command-line option), not the
    generator's."""
    from eden_gb300 import workloads
    gen, kw = (CASES[name][0], CASES[name][1]) if name in CASES else FULL_CASES[name][:2]
    kw = dict(kw)
    solver = kw.pop("cable_solver", "auto")
    spec = workloads.CONFIGS[gen](**kw)
    spec.cable_solver = solver
    return spec


# EDEN's extended loggers, added to the izh_net case's LEMS file: a trajectory
# window sampled every 1 ms, explicit sample points, and an ascii_v0 event
# file with a time window and a 10 ms heartbeat.  Their reference outputs are
# in tests/golden/loggers.npz.
LOGGER_FILES = ("sub.txt", "pts.txt", "ev.txt", "ev_id_time.txt")


def add_eden_loggers(lems_path):
    import re
    txt = open(lems_path).read()
    cols = re.findall(r'  <OutputColumn [^>]*/>\n', txt)[:3]
    # extended columns name their output units
    cols = [c.replace('/>', ' output_units="%s"/>' % u) for c, u in zip(cols, ("V", "mV", "mV"))]
    sels = re.findall(r'  <EventSelection [^>]*/>\n', txt)
    extra = (
        ' <EdenOutputFile id="sub" href="file://sub.txt" format="ascii_v0" starting_from="10ms" '
        'up_to_excluding="60.05ms" sampling_interval="1ms">\n' + "".join(cols) + ' </EdenOutputFile>\n'
        ' <EdenOutputFile id="pts" href="file://pts.txt" format="ascii_v0">\n'
        '  <SamplePoints><s t="0ms"/><s t="0.5ms"/><s t="12.34ms"/><s t="50ms"/><s t="99.95ms"/></SamplePoints>\n'
        + "".join(cols) + ' </EdenOutputFile>\n'
        ' <EdenEventOutputFile id="ev" href="file://ev.txt" format="ascii_v0" starting_from="5ms" '
        'up_to_excluding="80ms" maximum_interval="10ms">\n' + "".join(sels[:120]) + ' </EdenEventOutputFile>\n'
        ' <EdenEventOutputFile id="evi" href="file://ev_id_time.txt" format="ID_TIME">\n'
        + "".join(sels[100:160]) + ' </EdenEventOutputFile>\n')
    txt = txt.replace('</Simulation>', extra + '</Simulation>')
    open(lems_path, "w").write(txt)
