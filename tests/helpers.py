"""Shared helpers of the parity tests: workloads, scales and comparisons."""
import numpy as np

from oracle.parity import (cell_errors, error_statement, per_cell_bar, rel_err, total_scale,  # noqa: F401
                           truth_options)
from pflotran_gb300 import abi


def compare(net, gpu, ref, tol=1e-10, mask=None):
    """Max scaled relative errors of the parity outputs (GPU vs oracle)."""
    n = ref.ncells
    if mask is None:
        mask = np.ones(n, bool)
    out = {}
    out["pri_molal"] = rel_err(gpu.pri_molal.reshape(net.N, n), ref.pri_molal.reshape(net.N, n), 0.0)[:, mask].max()
    sc = total_scale(net, ref)
    out["total"] = rel_err(gpu.total_out.reshape(net.N, n), ref.total_out.reshape(net.N, n), sc)[:, mask].max()
    if net.Nm:
        k = np.array([mn.extra["k"] for mn in net.minerals])[:, None]
        area = ref.mnrl_area.reshape(-1, n)[:net.Nm]
        rs = k * area  # scale: rate constant x area
        out["mnrl_rate"] = rel_err(gpu.mnrl_rate.reshape(-1, n)[:net.Nm], ref.mnrl_rate.reshape(-1, n)[:net.Nm],
                                   rs)[:, mask].max()
        out["mnrl_volfrac"] = rel_err(gpu.mnrl_volfrac.reshape(-1, n)[:net.Nm],
                                      ref.mnrl_volfrac.reshape(-1, n)[:net.Nm], 1e-300)[:, mask].max()
    if net.Nix + net.Nsr:
        g = gpu.total_sorb_eq.reshape(net.N, n)
        r = ref.total_sorb_eq.reshape(net.N, n)
        s = np.maximum(np.abs(r).sum(0, keepdims=True) * 1e-6, 1e-300)
        out["total_sorb_eq"] = rel_err(g, r, s)[:, mask].max()
    out["ionic_strength"] = rel_err(gpu.ionic_strength, ref.ionic_strength, 0.0)[mask].max()
    if net.Nc and gpu.sec_molal is not None and ref.sec_molal is not None:
        # complexes below 1e-280 mol/kg are noise next to any total
        out["sec_molal"] = rel_err(gpu.sec_molal.reshape(-1, n)[:net.Nc], ref.sec_molal.reshape(-1, n)[:net.Nc],
                                   1e-280)[:, mask].max()
    return out


def constraint_problem(oracle, net, opt, cells, rows):
    """Constraint rows and per-cell values that describe each cell's own
    equilibrium state: rows maps component -> kind ('total', 'ph', 'log',
    'free', 'mineral:<k>', 'charge', 'gas:<k>' (partial pressure [bar]),
    'loggas:<k>' (its log10), 'sorb' (sorbed total)); unspecified components
    are 'total'.  Returns (types, spec ids, values[N, ncells])."""
    n, N = cells.ncells, net.N
    blocks = oracle.reaction_blocks(net.as_struct(), opt, cells.copy())
    m = cells.pri_molal.reshape(N, n)
    molar = m * (cells.den_kg * 1e-3)[None, :]
    types = np.full(N, abi.CONSTRAINT_TOTAL, np.int32)
    minerals = np.zeros(N, np.int32)
    values = blocks["total"].copy()
    for j, kind in rows.items():
        if kind == "ph":
            gp = np.array([oracle.activity_lag(net.as_struct(), float(I), N, net.Nc)[0][j] for I in cells.ionic_strength])
            types[j], values[j] = abi.CONSTRAINT_PH, -np.log10(m[j] * gp)
        elif kind == "log":
            types[j], values[j] = abi.CONSTRAINT_LOG, np.log10(molar[j])
        elif kind == "free":
            types[j], values[j] = abi.CONSTRAINT_FREE, molar[j]
        elif kind == "charge":
            types[j], values[j] = abi.CONSTRAINT_CHARGE_BAL, molar[j]
        elif kind.startswith("mineral:"):
            types[j], minerals[j], values[j] = abi.CONSTRAINT_MINERAL, int(kind.split(":")[1]), molar[j]
        elif kind.startswith(("gas:", "loggas:")):
            g = int(kind.split(":")[1])
            rx = net.gases[g - 1]
            act = np.array([oracle.activity_lag(net.as_struct(), float(I), N, net.Nc)[0] for I in cells.ionic_strength]).T
            lnQK = -rx.logK * 2.30258509299 + sum(nu * np.log(m[net.idx(q)] * act[net.idx(q)])
                                                 for q, nu in zip(rx.species, rx.stoich))
            p = np.exp(lnQK)
            types[j], minerals[j] = abi.CONSTRAINT_GAS, g
            values[j] = p if kind.startswith("gas:") else np.log10(p)
        elif kind == "sorb":
            types[j], values[j] = abi.CONSTRAINT_TOTAL_SORB, blocks["total_sorb"][j]
    return types, minerals, np.ascontiguousarray(values)


def gas_sorb_rows(net):
    """Constraint rows with GAS rows on a species of each of the network's
    gas reactions (the second in log10 form) and a TOTAL_SORB row on an
    exchanged cation; the rest TOTAL."""
    rows = {net.ionx[0]["ids"][1]: "sorb"}
    for g, rx in enumerate(net.gases):
        j = next(net.idx(q) for q in rx.species if net.idx(q) not in rows)
        rows[j] = ("gas:" if g == 0 else "loggas:") + str(g + 1)
    return rows


def truth_solve(oracle, net, opt, cells, dt, start, nthreads=None):
    """The root of the cells' equations (see oracle.parity.truth_solve)."""
    from oracle import parity
    return parity.truth_solve(net, opt, dt, cells, start, nthreads)
