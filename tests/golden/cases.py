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
}


def spec_of(name):
    from eden_gb300 import workloads
    gen, kw, _, _ = CASES[name]
    return workloads.CONFIGS[gen](**kw)
