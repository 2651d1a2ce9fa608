"""The GPU adjoint (edenGpuGrad*, eden_gb300/gradient.py) on ball-and-stick
cells: its forward trace against the plain simulation path, its gradients
against the double-precision oracle's forward-mode sensitivities and
central finite differences, independence of the checkpoint interval, the
torch.autograd form, and its error behaviour."""
import numpy as np
import pytest

from eden_gb300 import engine, lowering, workloads
from eden_gb300.gradient import CableGradient, per_cell_density_map
from oracle.cable_grad import Cable, loss_and_trace_grad

from test_cable_grad_oracle import K, driven_ball_and_stick, fd_grad_linear, per_cell_directions, small_ball_and_stick

pytestmark = pytest.mark.gpu

TRACE_ATOL_MV = 1e-3      # GPU forward vs the plain simulation path
# The FP32 adjoint against the FP64 forward sensitivities contracted with the
# same trace gradient, per parameter, relative to that parameter's largest
# gradient; against FP64 central differences (relative step 1e-4) of the same
# linear functional, which also carry the differences' truncation error.
GRAD_RTOL_TL = 1e-3
GRAD_RTOL_FD = 1e-3


def _case(n_inst=4, n_dend=20, length_ms=30.0, amp_na=0.5):
    spec, low, pm = small_ball_and_stick(n_inst, n_dend, length_ms, amp_na)
    rec = np.ascontiguousarray(low.phys_comp_off[:-1], np.int32)
    return spec, low, pm, rec


def _target(tr):
    return tr + 2.0 * np.sin(np.arange(len(tr)) * 0.01)[:, None]


def _close_per_param(g, ref, rtol):
    for j in range(K):
        scale = np.abs(ref[:, j]).max()
        np.testing.assert_allclose(g[:, j], ref[:, j], rtol=0, atol=rtol * scale, err_msg=f"parameter {j}")


def test_forward_matches_plain_simulation():
    _, low, pm, rec = _case()
    g = CableGradient(low, pm, rec_comp=rec)
    try:
        tr = g.forward(pm.values)
    finally:
        g.close()
    sim = engine.Simulation(low, mode=engine.MODE_PLAIN, trace_target=rec)
    try:
        rec_sim = sim.run()
    finally:
        sim.close()
    assert tr.shape == rec_sim.trace.shape
    assert tr.max() > 0.0
    np.testing.assert_allclose(tr, rec_sim.trace, rtol=0, atol=TRACE_ATOL_MV)


@pytest.mark.parametrize("amp_na", [-0.1, 0.5], ids=["subthreshold", "spiking"])
def test_gradient_matches_fp64_sensitivities_and_finite_differences(amp_na):
    """The gradient of an MSE loss of the GPU trace: the trace gradient it
    gives is contracted with the FP64 sensitivities and differentiated by
    FP64 central differences.  (Against the FP64 gradient of the MSE of the
    FP64 trace the spiking case differs by a few percent: float rounding
    moves spike times by a fraction of a step and the loss's trace gradient
    moves with them.)"""
    _, low, pm, rec = _case(amp_na=amp_na)
    cab = Cable(low, pm.chan_param, pm.cell_ra_param, low.phys_ra)
    tr64, dtr = cab.run(pm.values, low.n_steps, rec, per_cell_directions(pm.n_params))
    spiking = tr64.max() > 0.0
    assert spiking == (amp_na > 0.0)
    target = _target(tr64)
    g = CableGradient(low, pm, rec_comp=rec)
    try:
        tr = g.forward(pm.values)
        np.testing.assert_allclose(tr, tr64, rtol=0, atol=0.05 if spiking else 1e-3)
        _, tg = loss_and_trace_grad(tr.astype(np.float64), target)
        grad = g.backward(tg).reshape(-1, K)
    finally:
        g.close()
    g_tl = np.einsum("nc,jnc->cj", tg, dtr)
    _close_per_param(grad, g_tl, GRAD_RTOL_TL)
    g_fd = fd_grad_linear(cab, low, pm, rec, tg, 1e-4)
    _close_per_param(grad, g_fd, GRAD_RTOL_FD)


def test_checkpoint_interval_does_not_change_the_gradient():
    _, low, pm, rec = _case(n_inst=3, n_dend=10, length_ms=10.0)
    out = []
    for every in (7, 100, 1000):
        g = CableGradient(low, pm, rec_comp=rec, checkpoint_every=every)
        try:
            tr = g.forward(pm.values)
            out.append((tr, g.backward(np.sin(tr))))
        finally:
            g.close()
    for tr, gr in out[1:]:
        np.testing.assert_array_equal(tr, out[0][0])
        np.testing.assert_array_equal(gr, out[0][1])


def test_torch_autograd_matches_direct_calls():
    torch = pytest.importorskip("torch")
    _, low, pm, rec = _case(n_inst=3, n_dend=10, length_ms=10.0)
    g = CableGradient(low, pm, rec_comp=rec)
    try:
        p = torch.tensor(pm.values, device="cuda", requires_grad=True)
        tr = g.apply(p)
        target = torch.tensor(_target(tr.detach().cpu().numpy()), device="cuda")
        loss = ((tr - target) ** 2).mean()
        loss.backward()
        tg = (2.0 * (tr.detach() - target) / tr.numel()).cpu().numpy()
        direct = g.backward(tg)
        np.testing.assert_allclose(p.grad.cpu().numpy(), direct, rtol=1e-6, atol=0)
        # host tensors take the same path
        ph = torch.tensor(pm.values, requires_grad=True)
        trh = g.apply(ph)
        np.testing.assert_array_equal(trh.detach().numpy(), tr.detach().cpu().numpy())
    finally:
        g.close()


def test_gradient_of_unused_parameters_is_zero_and_no_ra_map_works():
    _, low, _, rec = _case(n_inst=2, n_dend=5, length_ms=5.0)
    pm = per_cell_density_map(low, [1], ra=False)   # soma gNa only
    pm.n_params += 3                                # three parameters nothing uses
    pm.values = np.concatenate([pm.values, np.ones(3, np.float32)])
    g = CableGradient(low, pm, rec_comp=rec)
    try:
        tr = g.forward(pm.values)
        gr = g.backward(np.ones_like(tr))
    finally:
        g.close()
    assert np.all(gr[-3:] == 0.0)
    assert np.all(gr[:2] != 0.0)


def test_errors():
    low = lowering.lower(workloads.multicomp_net(n_cells=4, in_degree=2, length_ms=1.0))
    pm = per_cell_density_map(low, [0], ra=False)
    with pytest.raises(engine.EdenGpuError) as e:
        CableGradient(low, pm)
    assert e.value.code == -1 and "Poisson" in str(e.value)
    # synapses from cells that spike: their events depend on the parameters
    low = lowering.lower(workloads.multicomp_net(n_cells=4, in_degree=2, length_ms=1.0, poisson_rate_hz=0.0))
    with pytest.raises(engine.EdenGpuError) as e:
        CableGradient(low, per_cell_density_map(low, [0], ra=False))
    assert e.value.code == -1 and "fixed in advance" in str(e.value)
    _, low, pm, rec = _case(n_inst=2, n_dend=5, length_ms=2.0)
    import dataclasses
    with pytest.raises(engine.EdenGpuError) as e:   # the adjoint follows the backward-Euler solve
        CableGradient(dataclasses.replace(low, cable_solver=lowering.CABLE_FWD_EULER), pm, rec_comp=rec)
    assert "backward-Euler" in str(e.value)
    g = CableGradient(low, pm, rec_comp=rec)
    try:
        with pytest.raises(engine.EdenGpuError) as e:
            g.backward(np.zeros((low.n_steps, len(rec))))   # no forward yet
        assert "edenGpuGradForward first" in str(e.value)
        bad = pm.values.copy()
        bad[K - 1] = -1.0                                   # a negative resistivity
        with pytest.raises(engine.EdenGpuError) as e:
            g.forward(bad)
        assert "must be positive" in str(e.value)
        g.forward(pm.values)                                # still usable
    finally:
        g.close()


@pytest.mark.parametrize("amp_na", [-0.05, 0.5], ids=["subthreshold", "spiking"])
def test_synaptic_weight_gradients(amp_na):
    """Gradients with respect to every synaptic weight (spike-list expTwo
    connections on the dendrite, timed expOne inputs on the soma) and the
    seven per-cell parameters, against the FP64 forward sensitivities
    contracted with the same trace gradient and against FP64 central
    differences of the same linear functional: per parameter kind, relative
    to that kind's largest gradient."""
    _, low, pm = driven_ball_and_stick(n_inst=3, n_dend=10, length_ms=30.0, amp_na=amp_na)
    rec = np.ascontiguousarray(low.phys_comp_off[:-1], np.int32)
    cab = Cable(low, pm.chan_param, pm.cell_ra_param, low.phys_ra, pm.syn_param, pm.timed_param)
    nw = len(pm.syn_param) + len(pm.timed_param)
    wpar = np.concatenate([pm.syn_param, pm.timed_param])
    dirs = np.zeros((K + nw, pm.n_params))
    dirs[:K] = per_cell_directions(pm.n_params)
    dirs[:K, -nw:] = 0.0
    dirs[K + np.arange(nw), wpar] = 1.0
    tr64, dtr = cab.run(pm.values, low.n_steps, rec, dirs)
    g = CableGradient(low, pm, rec_comp=rec)
    try:
        tr = g.forward(pm.values)
        np.testing.assert_allclose(tr, tr64, rtol=0, atol=0.05 if tr64.max() > 0 else 1e-3)
        _, tg = loss_and_trace_grad(tr.astype(np.float64), _target(tr64))
        grad = g.backward(tg)
    finally:
        g.close()
    ref_cell = np.einsum("nc,jnc->cj", tg, dtr[:K])
    _close_per_param(grad[:-nw].reshape(-1, K), ref_cell, GRAD_RTOL_TL)
    ref_w = np.einsum("nc,jnc->j", tg, dtr[K:])
    assert np.abs(ref_w).max() > 0.0
    np.testing.assert_allclose(grad[wpar], ref_w, rtol=0, atol=GRAD_RTOL_TL * np.abs(ref_w).max())
    h = 1e-4
    fd = np.zeros(nw)
    for j, p in enumerate(wpar):
        up = pm.values.astype(np.float64).copy()
        dn = up.copy()
        up[p] += h
        dn[p] -= h
        fd[j] = ((cab.run(up, low.n_steps, rec)[0] - cab.run(dn, low.n_steps, rec)[0]) * tg).sum() / (2 * h)
    np.testing.assert_allclose(grad[wpar], fd, rtol=0, atol=GRAD_RTOL_FD * np.abs(fd).max())


def test_synaptic_drive_forward_matches_plain_simulation():
    """The gradient path's forward with synaptic drive against the plain
    simulation path on the same model: the same spikes and potentials to the
    rounding of the synapses' event-driven sums."""
    _, low, pm = driven_ball_and_stick(n_inst=4, n_dend=10, length_ms=40.0)
    rec = np.ascontiguousarray(low.phys_comp_off[:-1], np.int32)
    g = CableGradient(low, pm, rec_comp=rec)
    try:
        tr = g.forward(pm.values)
    finally:
        g.close()
    sim = engine.Simulation(low, mode=engine.MODE_PLAIN, trace_target=rec)
    try:
        ref = sim.run()
    finally:
        sim.close()
    assert tr.max() > 0.0
    np.testing.assert_allclose(tr, ref.trace, rtol=0, atol=0.05)
