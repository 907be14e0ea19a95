"""The Newton Jacobian (CPU, oracle): the exact option is the derivative of
RReact's residual; the reference's own Jacobian is not, which is why its
Newton iteration converges linearly on networks with surface complexation
and precipitating minerals."""
import numpy as np

from pflotran_gb300 import abi, workloads


def _fd_contraction(oracle, net, opt, cells, dt, k, m):
    """Spectral radius of I - J^-1 J_fd in ln m (the Newton contraction
    factor near the root) and the max column-scaled Jacobian error."""
    ns = net.as_struct()
    _, J = oracle.newton_system(ns, opt, dt, cells, k, m)
    N = net.N
    Jfd = np.zeros((N, N))
    for j in range(N):
        h = 1e-6 * m[j]
        mp, mm = m.copy(), m.copy()
        mp[j] += h
        mm[j] -= h
        Jfd[:, j] = (oracle.newton_system(ns, opt, dt, cells, k, mp)[0] -
                     oracle.newton_system(ns, opt, dt, cells, k, mm)[0]) / (2 * h)
    A, B = J * m[None, :], Jfd * m[None, :]
    rho = np.abs(np.linalg.eigvals(np.linalg.solve(A, B) - np.eye(N))).max()
    return rho


def test_exact_jacobian_is_the_derivative(oracle):
    net, opt, cells, dt = workloads.synthetic_cells(40, seed=21)
    sol = cells.copy()
    oracle.react(net.as_struct(), opt, dt, sol, 0, 4)
    exact = workloads.default_options(use_isothermal=1, jacobian=abi.JACOBIAN_EXACT)
    rho_ref, rho_exact = [], []
    for k in range(cells.ncells):
        if sol.status[k] != 0:
            continue
        m = sol.pri_molal.reshape(net.N, -1)[:, k].copy()
        rho_ref.append(_fd_contraction(oracle, net, opt, cells, dt, k, m))
        rho_exact.append(_fd_contraction(oracle, net, exact, cells, dt, k, m))
    rho_ref, rho_exact = np.array(rho_ref), np.array(rho_exact)
    assert rho_exact.max() < 1e-5, rho_exact.max()          # finite-difference noise only
    assert np.median(rho_ref) > 1e-3 and rho_ref.max() > 0.1  # linear convergence


def test_exact_jacobian_same_root_fewer_iterations(oracle):
    net, opt, cells, dt = workloads.synthetic_cells(1000, seed=22)
    a, b = cells.copy(), cells.copy()
    oracle.react(net.as_struct(), opt, dt, a, 0, 4)
    exact = workloads.default_options(use_isothermal=1, jacobian=abi.JACOBIAN_EXACT)
    oracle.react(net.as_struct(), exact, dt, b, 0, 4)
    ok = (a.status == 0) & (b.status == 0)
    assert ok.mean() > 0.99
    rel = np.abs(b.pri_molal - a.pri_molal) / a.pri_molal
    assert np.percentile(rel.reshape(net.N, -1)[:, ok].max(0), 99) < 1e-10
    assert rel.reshape(net.N, -1)[:, ok].max() < 1e-8
    assert b.iterations[ok].mean() < 0.75 * a.iterations[ok].mean()
    assert b.iterations.max() < 200


def _fd_blocks(oracle, net, opt, cells, k, key_v, h_rel=1e-6):
    """Central finite differences of output `key_v` of the oracle's reaction
    blocks with respect to the free-ion molalities of cell k."""
    N = net.N
    one = cells.subset(np.array([k]), net)
    base = one.copy()
    fd = np.zeros((N, N))
    for j in range(N):
        vals = []
        for sgn in (1.0, -1.0):
            c = base.copy()
            m = c.pri_molal.copy()
            h = h_rel * m[j]
            m[j] += sgn * h
            c.pri_molal = m
            vals.append(oracle.reaction_blocks(net.as_struct(), opt, c)[key_v][:, 0])
        fd[:, j] = (vals[0] - vals[1]) / (2 * h_rel * base.pri_molal[j])
    return fd


def test_reaction_blocks_are_derivatives(oracle):
    """Global-implicit blocks: d total/dm and d total_sorb/dm are the
    derivatives of the totals (surface complexation exact only with the exact
    option); the reaction Jacobian is that of the reaction residual up to
    RKineticMineral's den/1000 factor (exact with the option)."""
    net, opt, cells, dt = workloads.synthetic_cells(6, seed=23)
    sol = cells.copy()
    oracle.react(net.as_struct(), opt, dt, sol, 0, 2)
    exact = workloads.default_options(use_isothermal=1, jacobian=abi.JACOBIAN_EXACT)
    rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()
    for k in range(cells.ncells):
        if sol.status[k] != 0:
            continue
        one = sol.subset(np.array([k]), net)
        bx = oracle.reaction_blocks(net.as_struct(), exact, one.copy())
        br = oracle.reaction_blocks(net.as_struct(), opt, one.copy())
        # blocks are [cell, j, i]: transpose to [i, j]
        assert rel(bx["dtotal"][0].T, _fd_blocks(oracle, net, exact, sol, k, "total")) < 1e-6
        assert rel(bx["dtotal_sorb"][0].T, _fd_blocks(oracle, net, exact, sol, k, "total_sorb")) < 1e-6
        fd_r = _fd_blocks(oracle, net, exact, sol, k, "res")
        if np.abs(fd_r).max() > 0:
            assert rel(bx["jac"][0].T, fd_r) < 1e-5
        # the reference's aqueous block is exact, its sorbed and reaction blocks are not
        assert rel(br["dtotal"][0].T, bx["dtotal"][0].T) < 1e-12
        np.testing.assert_array_equal(br["res"], bx["res"])


def test_exact_jacobian_is_the_derivative_with_rate_prefactors(oracle):
    """Minerals with rate prefactors (Monod terms in primaries and in an
    aqueous complex, a prefactor with its own activation energy,
    reaction_mineral.F90:743-782): the exact option's Jacobian, including
    the prefactor terms of :897-997, is the derivative of the residual."""
    net, opt, cells, dt = workloads.synthetic_cells(30, seed=24)
    workloads.add_rate_prefactors(net)
    sol = cells.copy()
    oracle.react(net.as_struct(), opt, dt, sol, 0, 4)
    exact = workloads.default_options(use_isothermal=1, jacobian=abi.JACOBIAN_EXACT)
    rho = []
    for k in range(cells.ncells):
        if sol.status[k] != 0:
            continue
        m = sol.pri_molal.reshape(net.N, -1)[:, k].copy()
        rho.append(_fd_contraction(oracle, net, exact, cells, dt, k, m))
    assert len(rho) >= 25 and max(rho) < 1e-5, max(rho)
