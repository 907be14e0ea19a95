"""Error metrics of GPU results against the oracle (test infrastructure).

Used by tests/ and by bench.py's CPU-baseline leg, never by the library.

Scaled relative error |x - y| / max(|y|, s), with s the magnitude of the
terms a quantity is made of: for an aqueous total den_L*(m_j + sum_i
|nu_ij| C_i), for a mineral rate the rate constant x area, for a volume
fraction nothing (plain relative).  The bar is 1e-10.
"""
import numpy as np


def rel_err(x, y, scale):
    # the 1e-300 floor keeps 0/0 (an absent mineral's zero rate) at 0
    return np.abs(x - y) / np.maximum(np.maximum(np.abs(y), scale), 1e-300)


def _nu(net):
    """Stoichiometric matrix (Nc x N) of the aqueous complexes, from the tables."""
    t = net._tables if net._tables is not None else net.build()
    nu = np.zeros((net.Nc, net.N))
    ld = t["eqcplx_ld"]
    ids = t["eqcplxspecid"].reshape(-1, ld + 1)
    st = t["eqcplxstoich"].reshape(-1, ld)
    for i in range(net.Nc):
        for k in range(ids[i, 0]):
            nu[i, ids[i, k + 1] - 1] = st[i, k]
    return nu


def total_scale(net, cells):
    """Per-component magnitude of the aqueous total: den_L*(m_j + sum_i |nu_ij| C_i)."""
    n = cells.ncells
    m = cells.pri_molal.reshape(net.N, n)
    if net.Nc:
        C = cells.sec_molal.reshape(-1, n)[:net.Nc]
        s = m + np.abs(_nu(net)).T @ C
    else:
        s = m.copy()
    return s * (cells.den_kg * 1e-3)[None, :]


def cell_errors(net, x, y):
    """Per-cell scaled relative errors of x against y (max over the
    components) for the aqueous totals, mineral volume fractions and mineral
    rates."""
    n = y.ncells
    errs = {"total": rel_err(x.total_out.reshape(net.N, n), y.total_out.reshape(net.N, n), total_scale(net, y))}
    if net.Nm:
        k = np.array([mn.extra["k"] for mn in net.minerals])[:, None]
        area = y.mnrl_area.reshape(-1, n)[:net.Nm]
        errs["mnrl_rate"] = rel_err(x.mnrl_rate.reshape(-1, n)[:net.Nm], y.mnrl_rate.reshape(-1, n)[:net.Nm], k * area)
        errs["mnrl_volfrac"] = rel_err(x.mnrl_volfrac.reshape(-1, n)[:net.Nm], y.mnrl_volfrac.reshape(-1, n)[:net.Nm],
                                       1e-300)
    return {q: e.max(axis=0) for q, e in errs.items()}


def error_statement(net, x, y, mask=None):
    """Max and 99th percentile over the cells in `mask` of `cell_errors`."""
    errs = cell_errors(net, x, y)
    if mask is None:
        mask = np.ones(y.ncells, bool)
    if not mask.any():
        return {q: {"max": None, "p99": None} for q in errs}
    return {q: {"max": float(e[mask].max()), "p99": float(np.percentile(e[mask], 99))} for q, e in errs.items()}


def truth_options(opt):
    """Options of the reference root: the same equations solved with the exact
    Jacobian, no damping, to a 1e-16 relative residual."""
    from pflotran_gb300 import abi
    o = abi.Options.from_buffer_copy(opt)
    o.jacobian = abi.JACOBIAN_EXACT
    o.exact_jacobian_after = 1
    o.residual_tol_kind = abi.RESIDUAL_RELATIVE
    o.max_residual_tolerance = 1e-16
    o.max_relative_change_tolerance = 0.0
    o.max_iterations = 1000
    return o


def solve(net, opt, dt, cells, precision=0, nthreads=None, alt_guess=None):
    """The oracle's RReact on a copy of a host CellBatch (outputs allocated)."""
    import os

    from . import oracle
    t = cells.copy()
    n = cells.ncells
    if t.sec_molal is None:
        t.sec_molal = np.zeros(max(net.Nc, 1) * n)
    if t.total_out is None:
        t.total_out = np.zeros(net.N * n)
    if t.mnrl_rate is None:
        t.mnrl_rate = np.zeros(max(net.Nm, 1) * n)
    t.iterations = np.zeros(n, np.int32)
    t.status = np.zeros(n, np.int32)
    t.alt_guess = None if alt_guess is None else np.ascontiguousarray(alt_guess, np.float64)
    oracle.react(net.as_struct(), opt, dt, t, precision, nthreads or os.cpu_count() or 1)
    return t


def truth_solve(net, opt, dt, cells, start, nthreads=None):
    """The root of the cells' equations, solved by the oracle's long-double
    instantiation to a 1e-16 relative residual (binary128 on aarch64, 80-bit
    extended on x86-64) with undamped exact Newton from `start`'s free-ion
    molalities (a converged double solution of the same cells, so a few
    quadratically convergent iterations).  Any Newton path that stops at the
    1e-12 test lands within the tolerance x the cell's conditioning of it."""
    return solve(net, truth_options(opt), dt, cells, precision=1, nthreads=nthreads, alt_guess=start.pri_molal)


def per_cell_bar(net, x, ref, truth, tol=1e-10, mask=None, alt=None):
    """Per cell and quantity (totals, volume fractions, rates): x is within
    `tol` of the oracle `ref`, or no farther from the root `truth` than `ref`
    itself is (floor `tol`), or -- given `alt`, the oracle's answer for the
    same cell from another starting guess -- no farther from `ref` than
    `alt` is.  The second and third branches cover ill-conditioned cells,
    where two Newton paths that both stop at the 1e-12 residual test (a
    rounding difference in the stopping iteration, a different starting
    guess) land up to the tolerance x the conditioning apart: the third
    measures that spread on the oracle itself.  Returns {quantity: (pass
    mask, errors vs ref, errors vs truth, ref vs truth)}; cells outside
    `mask` pass."""
    exr, ext, ert = cell_errors(net, x, ref), cell_errors(net, x, truth), cell_errors(net, ref, truth)
    spread = cell_errors(net, alt, ref) if alt is not None else None
    if mask is None:
        mask = np.ones(ref.ncells, bool)
    out = {}
    for q in exr:
        ok = (exr[q] <= tol) | (ext[q] <= np.maximum(tol, ert[q]))
        if spread is not None:
            ok |= exr[q] <= spread[q]
        out[q] = (ok | ~mask, exr[q], ext[q], ert[q])
    return out


def bar_failures(net, x, ref, truth, bar, alt=None):
    """The cells a per_cell_bar result fails, one line each: quantity, cell,
    errors vs the oracle / x vs root / oracle vs root (/ oracle spread),
    iterations of x and of the oracle."""
    spread = cell_errors(net, alt, ref) if alt is not None else None
    lines = []
    for q, (ok, exr, ext, ert) in bar.items():
        for c in np.flatnonzero(~ok):
            s = f" spread {spread[q][c]:.3e}" if spread is not None else ""
            lines.append(f"{q} cell {c}: vs oracle {exr[c]:.3e}, vs root {ext[c]:.3e}, oracle vs root "
                         f"{ert[c]:.3e}{s}, iterations {int(x.iterations[c])}/{int(ref.iterations[c])}")
    return lines
