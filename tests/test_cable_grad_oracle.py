"""The double-precision cable oracle that checks the GPU adjoint: its
forward run against the double-precision C restatement of the reference
(libeden_port64), and its forward-mode sensitivities against central
finite differences of its own forward run.  CPU only."""
import numpy as np
import pytest

from eden_gb300 import lowering, workloads
from eden_gb300.gradient import per_cell_density_map, with_weights
from oracle.cable_grad import Cable, loss_and_trace_grad
from oracle.port import eden_port

# the seven per-instance parameters of the ball-and-stick workload: soma gNa,
# gK, gL, dendrite gNa, gK, gL (their channelDensity indices), then Ra
BS_DENSITIES = [1, 2, 0, 4, 5, 3]
K = 7


def small_ball_and_stick(n_inst=3, n_dend=8, length_ms=20.0, amp_na=0.5):
    spec = workloads.ball_and_stick(n_inst=n_inst, n_dend=n_dend, length_ms=length_ms, amp_na=amp_na)
    low = lowering.lower(spec)
    return spec, low, per_cell_density_map(low, BS_DENSITIES)


def per_cell_directions(n_params):
    d = np.zeros((K, n_params))
    for j in range(K):
        d[j, j::K] = 1.0
    return d


def fd_grad(cab, low, pm, rec, target, h):
    """Per-cell central differences of the MSE with relative step h."""
    g = np.zeros((len(rec), K))
    n = target.size
    for j in range(K):
        up = pm.values.astype(np.float64).copy()
        dn = up.copy()
        up[j::K] *= 1 + h
        dn[j::K] *= 1 - h
        tu, _ = cab.run(up, low.n_steps, rec)
        td, _ = cab.run(dn, low.n_steps, rec)
        g[:, j] = (((tu - target) ** 2).sum(0) - ((td - target) ** 2).sum(0)) / n / (2 * h * pm.values[j::K])
    return g


def fd_grad_linear(cab, low, pm, rec, w, h):
    """Per-cell central differences of sum(w * trace) with relative step h."""
    g = np.zeros((len(rec), K))
    for j in range(K):
        up = pm.values.astype(np.float64).copy()
        dn = up.copy()
        up[j::K] *= 1 + h
        dn[j::K] *= 1 - h
        tu, _ = cab.run(up, low.n_steps, rec)
        td, _ = cab.run(dn, low.n_steps, rec)
        g[:, j] = ((tu - td) * w).sum(0) / (2 * h * pm.values[j::K])
    return g


def test_param_map_reproduces_the_workload_parameters():
    spec, low, pm = small_ball_and_stick()
    np.testing.assert_allclose(pm.values.reshape(-1, K), spec.params, rtol=1e-6)


def test_forward_matches_double_precision_port():
    _, low, pm = small_ball_and_stick()
    rec = low.phys_comp_off[:-1]
    cab = Cable(low, pm.chan_param, pm.cell_ra_param, low.phys_ra)
    tr, _ = cab.run(pm.values, low.n_steps, rec)
    ref = eden_port.run(low, trace_target=rec, double=True)["trace"]
    assert tr.max() > 0.0          # the cells spike
    # the port returns its double trace rounded to float
    np.testing.assert_allclose(tr, ref, rtol=0, atol=2e-5)


def test_sensitivities_match_finite_differences():
    _, low, pm = small_ball_and_stick()
    rec = low.phys_comp_off[:-1]
    cab = Cable(low, pm.chan_param, pm.cell_ra_param, low.phys_ra)
    tr, dtr = cab.run(pm.values, low.n_steps, rec, per_cell_directions(pm.n_params))
    target = tr + 0.5 * np.sin(np.arange(len(tr)))[:, None]
    _, tg = loss_and_trace_grad(tr, target)
    g_tl = np.einsum("nc,jnc->cj", tg, dtr)
    # a small step isolates the derivative ...
    g_fd = fd_grad(cab, low, pm, rec, target, 1e-6)
    np.testing.assert_allclose(g_tl, g_fd, rtol=1e-4, atol=1e-6 * np.abs(g_fd).max())
    # ... and the 1e-4 relative step agrees to its truncation error
    g_fd4 = fd_grad(cab, low, pm, rec, target, 1e-4)
    assert np.abs(g_tl - g_fd4).max() <= 1e-3 * np.abs(g_fd4).max()


def test_oracle_refuses_networks_whose_synaptic_events_are_not_fixed():
    # Poisson inputs and synapses from cells that spike
    low = lowering.lower(workloads.multicomp_net(n_cells=4, in_degree=2, length_ms=1.0))
    with pytest.raises(ValueError):
        Cable(low, None)
    low = lowering.lower(workloads.multicomp_net(n_cells=4, in_degree=2, length_ms=1.0, poisson_rate_hz=0.0))
    with pytest.raises(ValueError):
        Cable(low, None).run(per_cell_density_map(low, [0], ra=False).values, 4, [0])


def driven_ball_and_stick(n_inst=3, n_dend=8, length_ms=20.0, amp_na=0.5, syn_drive=4):
    """Ball-and-stick cells with synaptic drive fixed in advance (spike-list
    connections onto the dendrite, timed inputs onto the soma) and one
    parameter per synaptic weight after the seven per cell."""
    spec = workloads.ball_and_stick(n_inst=n_inst, n_dend=n_dend, length_ms=length_ms, amp_na=amp_na,
                                    syn_drive=syn_drive)
    low = lowering.lower(spec)
    return spec, low, with_weights(low, per_cell_density_map(low, BS_DENSITIES))


@pytest.mark.parametrize("amp_na", [-0.05, 0.5], ids=["subthreshold", "spiking"])
def test_synaptic_drive_matches_double_precision_port(amp_na):
    """The drive's conductances (expTwo and expOne, spike-list connections
    and timed inputs) against the double-precision C restatement."""
    _, low, pm = driven_ball_and_stick(amp_na=amp_na)
    rec = low.phys_comp_off[:-1]
    cab = Cable(low, pm.chan_param, pm.cell_ra_param, low.phys_ra, pm.syn_param, pm.timed_param)
    tr, _ = cab.run(pm.values, low.n_steps, rec)
    ref = eden_port.run(low, trace_target=rec, double=True)
    assert ref["rc"] == 0
    np.testing.assert_allclose(tr, ref["trace"], rtol=0, atol=2e-5)
    meta, ghat = cab.drive(low.n_steps)
    assert len(meta) == len(low.syn_target) + len(low.timed_target) and ghat.max() > 0.0


def test_weight_sensitivities_match_finite_differences():
    _, low, pm = driven_ball_and_stick()
    rec = low.phys_comp_off[:-1]
    cab = Cable(low, pm.chan_param, pm.cell_ra_param, low.phys_ra, pm.syn_param, pm.timed_param)
    w = np.concatenate([pm.syn_param, pm.timed_param])
    dirs = np.zeros((len(w), pm.n_params))
    dirs[np.arange(len(w)), w] = 1.0
    tr, dtr = cab.run(pm.values, low.n_steps, rec, dirs)
    tg = np.sin(np.arange(tr.size)).reshape(tr.shape) / tr.size
    g_tl = np.einsum("nc,jnc->j", tg, dtr)
    h = 1e-4
    g_fd = np.zeros(len(w))
    for j, p in enumerate(w):
        up = pm.values.astype(np.float64).copy()
        dn = up.copy()
        up[p] += h
        dn[p] -= h
        g_fd[j] = ((cab.run(up, low.n_steps, rec)[0] - cab.run(dn, low.n_steps, rec)[0]) * tg).sum() / (2 * h)
    np.testing.assert_allclose(g_tl, g_fd, rtol=1e-4, atol=1e-5 * np.abs(g_fd).max())
    assert np.abs(g_tl).max() > 0.0
