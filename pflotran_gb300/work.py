"""Algorithmic work and traffic of one reaction step (roofline numerators).

Flops follow the counting convention: +, -, *, /, sqrt = 1 flop, an FMA =
2 flops, exp/log/pow = 1 flop (and also counted separately as
transcendentals).  The count is that of RReact's algorithm per Newton
iteration on the given network -- RTotal, the sorption models, the
accumulation terms, RKineticMineral, RSolve (ludcmp/lubksb) and the update --
not of any particular implementation of it.  Ion-exchange inner Newton
loops are counted at 3 inner iterations per reaction and Newton iteration.
"""
from __future__ import annotations

import numpy as np


def per_iteration(net):
    t = net._tables if net._tables is not None else net.build()
    N = net.N
    fl = 0
    tr = 0
    fl += N  # ln a = ln m + ln gamma
    ld = t["eqcplx_ld"]
    ids = t["eqcplxspecid"].reshape(-1, ld + 1)
    for i in range(net.Nc):
        z = int(ids[i, 0])
        fl += 2 * z      # lnQK
        tr += 1          # exp
        fl += 1          # / gamma
        fl += 2 * z      # totals
        fl += z + 2 * z * z  # dPsi/dm
    fl += N + N * N      # molality -> molarity for totals and derivatives
    fl += 2 * N + N * N  # accumulation residual and Jacobian
    # ion exchange
    ldx = t["eqionx_ld"]
    xid = t["eqionx_rxn_cationid"].reshape(-1, ldx + 1)
    for r in range(net.Nix):
        z = int(xid[r, 0])
        fl += 3 * (z * 6 + 4)
        tr += 3 * (z - 1)
        fl += 2 * z + z * z * 4
    # surface complexation
    lds = t["srfcplx_ld"]
    sid = t["srfcplxspecid"].reshape(-1, lds + 1)
    for r in range(net.Nsr):
        for k in net.srfrxn[r]["complexes"]:
            z = len(k.species)
            fl += 2 * 2 * z + 4
            tr += 2
            fl += 2 * z + 3 * z + 2 * z * z
        fl += 6
    if net.Nix + net.Nsr:
        fl += 2 * N + N * N
    # kinetic minerals
    ldm = t["kinmnrl_ld"]
    mid = t["kinmnrlspecid"].reshape(-1, ldm + 1)
    for m in range(net.Nm):
        z = int(mid[m, 0])
        fl += 2 * z + 8 + 2 * z + 3 * z + 2 * z * z
        tr += 1
    # RSolve: row scaling, log-column scaling, LU with pivot scaling, solve
    fl += N * N + N + N * N
    fl += int(round(2 * N ** 3 / 3)) + N * N // 2 + N
    fl += 2 * N * N + N
    # update: clamp, exp, product, relative change
    fl += 4 * N
    tr += N
    return fl + tr, tr


def per_cell_setup(net, isothermal=True):
    N = net.N
    fl = 3 * N + 10
    tr = N
    if not isothermal:
        fl += 8 * (net.Nc + net.Nm + net.Nsc)
        tr += 1
    fl += 8 * (N + net.Nc)  # activity coefficients
    tr += N + net.Nc
    return fl + tr, tr


def step_flops(net, iterations, isothermal=True):
    """Algorithmic flops of one step given per-cell iteration counts."""
    fi, _ = per_iteration(net)
    fs, _ = per_cell_setup(net, isothermal)
    return float(np.sum(iterations, dtype=np.float64)) * fi + len(iterations) * fs


def bytes_per_cell(net, with_sec_molal=False):
    """HBM bytes one cell moves: every input and state array read once, every
    state and output array written once."""
    N, Nm = net.N, net.Nm
    sorb = net.Nix + net.Nsr > 0
    rd = 6 + N + N + 1 + 2 * Nm + (N if sorb else 0) + net.Nix + net.Nsr  # inputs + state in
    wr = N + 1 + Nm + (N if sorb else 0) + net.Nix + net.Nsr + N + Nm   # state out + totals + rates
    if with_sec_molal:
        wr += net.Nc
    return 8 * (rd + wr) + 8  # + iterations and status
