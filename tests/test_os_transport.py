"""Transport stand-in of the time-stepped run (CPU): permeability field,
Darcy fluxes and upwind advection."""
import pytest

torch = pytest.importorskip("torch")

from pflotran_gb300 import os_run


def _flow(shape=(12, 10, 8), seed=4):
    K = os_run.lognormal_permeability(shape, 1.5, 3.0, seed, "cpu")
    qx, qy, qz, its = os_run.darcy_fluxes(K, rtol=1e-12)
    return K, qx, qy, qz, its


def test_permeability_field_statistics():
    K = os_run.lognormal_permeability((32, 32, 32), 1.5, 4.0, 1, "cpu")
    g = torch.log(K)
    assert abs(float(g.mean())) < 1e-10
    assert abs(float(g.std()) - 1.5) < 1e-10
    # correlation decays with lag along each axis
    c = lambda k: float(((g - g.mean()) * (torch.roll(g, k, 0) - g.mean())).mean() / g.var())
    assert c(1) > c(4) > c(12)
    assert c(1) > 0.5


def test_darcy_fluxes_are_divergence_free():
    K, qx, qy, qz, its = _flow()
    net = (qx[:-1] - qx[1:]) + (qy[:, :-1] - qy[:, 1:]) + (qz[:, :, :-1] - qz[:, :, 1:])
    scale = float(qx.abs().max())
    assert float(net.abs().max()) < 1e-9 * scale
    assert float((qx[0].sum() - qx[-1].sum()).abs()) < 1e-9 * float(qx[0].sum())
    assert float(qx[0].min()) > 0  # head drop drives flow into the west face


def test_upwind_preserves_uniform_state_and_balances_mass():
    K, qx, qy, qz, _ = _flow()
    por = 0.25
    out = float(os_run.outflow_rate(qx, qy, qz).max())
    dt = 0.9 * por / out  # CFL-limited
    # uniform water with the same inflow stays uniform
    T = torch.full((3,) + K.shape, 2.0, dtype=torch.float64)
    T[1] = 5.0
    inflow = torch.tensor([2.0, 5.0, 2.0], dtype=torch.float64)
    T1 = os_run.upwind_advect(T, qx, qy, qz, por, dt, inflow)
    assert float((T1 - T).abs().max()) < 1e-9
    # a front: resident water 0, inflow 1; mass change equals net boundary flux
    T = torch.zeros((1,) + K.shape, dtype=torch.float64)
    inflow = torch.tensor([1.0], dtype=torch.float64)
    for _ in range(20):
        Tn = os_run.upwind_advect(T, qx, qy, qz, por, dt, inflow)
        dm = float((Tn - T).sum()) * por
        flux = dt * (float(qx[0].sum()) * 1.0 - float((qx[-1] * T[0, -1]).sum()))
        assert abs(dm - flux) < 1e-10 * max(1.0, abs(flux))
        T = Tn
        assert float(T.min()) >= -1e-15 and float(T.max()) <= 1.0 + 1e-12  # monotone under CFL
    assert float(T[0, 0].mean()) > float(T[0, -1].mean())


def test_transport_library_exports_the_upwind_step():
    import ctypes
    lib = os_run._transport()
    assert isinstance(lib.pfchem_transport_upwind, ctypes._CFuncPtr)


def test_upwind_weights_reproduce_the_flux_form():
    """T' = a0 T + sum_f a_f T_f with the per-cell weights equals the flux
    form to rounding; the weights are non-negative under the CFL limit and
    sum (with the outflow) to one."""
    K, qx, qy, qz, _ = _flow()
    por = 0.25
    dt = 0.9 * por / float(os_run.outflow_rate(qx, qy, qz).max())
    a = os_run.upwind_coefficients(qx, qy, qz, por, dt)
    assert a.shape == (7,) + K.shape
    assert float(a.min()) >= 0.0
    g = torch.Generator().manual_seed(2)
    T = torch.rand((3,) + K.shape, dtype=torch.float64, generator=g)
    inflow = torch.tensor([0.5, 2.0, 1.0], dtype=torch.float64)
    nb = torch.zeros((6,) + T.shape, dtype=torch.float64)
    nb[0, :, 1:] = T[:, :-1]
    nb[0, :, 0] = inflow[:, None, None]
    nb[1, :, :-1] = T[:, 1:]
    nb[2, :, :, 1:] = T[:, :, :-1]
    nb[3, :, :, :-1] = T[:, :, 1:]
    nb[4, :, :, :, 1:] = T[:, :, :, :-1]
    nb[5, :, :, :, :-1] = T[:, :, :, 1:]
    out = a[0] * T + (a[1:, None] * nb).sum(0)
    ref = os_run.upwind_advect(T, qx, qy, qz, por, dt, inflow)
    assert float((out - ref).abs().max()) <= 1e-14 * float(ref.abs().max())
