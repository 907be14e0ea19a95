"""ctypes loader for the CPU oracle (test infrastructure only).

The oracle restates PFLOTRAN's per-cell reaction step in C++
(oracle/pfchem_oracle.cpp).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs use it, as the checker; the GPU library never
calls it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libpfchem_oracle.so")
_lib = None


def build(force=False):
    if force or not os.path.exists(_LIB) or (
            os.path.getmtime(_LIB) < os.path.getmtime(os.path.join(_HERE, "pfchem_oracle.cpp"))):
        subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(_LIB)
        l.pfo_react_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_int, C.c_int]
        l.pfo_react_batch.restype = C.c_int
        l.pfo_speciate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        l.pfo_activity_lag.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
        l.pfo_rsolve.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        l.pfo_fit_logK.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        l.pfo_interpolate_logK.argtypes = [C.c_void_p, C.c_double]
        l.pfo_interpolate_logK.restype = C.c_double
        l.pfo_ifc67_density.argtypes = [C.c_double, C.c_double]
        l.pfo_equilibrate_constraints.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        l.pfo_update_mineral_properties.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        l.pfo_reaction_blocks.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        l.pfo_newton_system.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_int64, C.c_void_p,
                                        C.c_void_p, C.c_void_p]
        l.pfo_ifc67_density.restype = C.c_double
        _lib = l
    return _lib


def react(net_struct, opt, dt, cells, precision=0, nthreads=None):
    """Runs the restated RReact on a host CellBatch in place."""
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    s = cells.struct()
    assert s.on_device == 0
    return lib().pfo_react_batch(C.byref(net_struct), C.byref(opt), dt, C.byref(s), precision, nthreads)


def speciate(net_struct, opt, cells):
    s = cells.struct()
    return lib().pfo_speciate(C.byref(net_struct), C.byref(opt), C.byref(s))


def ifc67_density(t, p):
    return lib().pfo_ifc67_density(t, p)


def fit_logK(temps, logK):
    t = np.ascontiguousarray(temps, np.float64)
    k = np.ascontiguousarray(logK, np.float64)
    out = np.zeros(5)
    r = lib().pfo_fit_logK(len(t), t.ctypes.data, k.ctypes.data, out.ctypes.data)
    if r:
        raise RuntimeError("singular log K fit")
    return out


def interpolate_logK(coefs, temp):
    c = np.ascontiguousarray(coefs, np.float64)
    return lib().pfo_interpolate_logK(c.ctypes.data, temp)


def activity_lag(net_struct, I, N, Nc):
    gp = np.zeros(max(N, 1))
    gc = np.zeros(max(Nc, 1))
    lib().pfo_activity_lag(C.byref(net_struct), I, gp.ctypes.data, gc.ctypes.data)
    return gp[:N], gc[:Nc]


def equilibrate_constraint(net_struct, opt, cells, types, conc):
    """Constraint speciation of the single cell in `cells` (host CellBatch)."""
    l = lib()
    l.pfo_equilibrate_constraint.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    t = np.ascontiguousarray(types, np.int32)
    c = np.ascontiguousarray(conc, np.float64)
    it = np.zeros(1, np.int32)
    s = cells.struct()
    r = l.pfo_equilibrate_constraint(C.byref(net_struct), C.byref(opt), C.byref(s), t.ctypes.data,
                                     c.ctypes.data, it.ctypes.data)
    if r:
        raise RuntimeError(f"constraint equilibration failed ({r})")
    return int(it[0])


def newton_system(net_struct, opt, dt, cells, k, m):
    """RReact's residual F and Jacobian dF/dm (N x N) for cell k at molalities m."""
    import numpy as np
    N = len(m)
    m = np.ascontiguousarray(m, np.float64)
    F = np.zeros(N)
    J = np.zeros(N * N)
    s = cells.struct()
    r = lib().pfo_newton_system(C.byref(net_struct), C.byref(opt), dt, C.byref(s), k, m.ctypes.data, F.ctypes.data,
                                J.ctypes.data)
    if r:
        raise RuntimeError("pfo_newton_system failed")
    return F, J.reshape(N, N)


def reaction_blocks(net_struct, opt, cells):
    """Global-implicit per-cell blocks of a host CellBatch (see pfo_reaction_blocks):
    dict of numpy arrays shaped like ReactionStep.reaction_blocks'."""
    import numpy as np
    from pflotran_gb300 import abi
    n = cells.ncells
    N = cells.pri_molal.size // n
    out = {"res": np.zeros((N, n)), "total": np.zeros((N, n)), "total_sorb": np.zeros((N, n)),
           "jac": np.zeros((n, N, N)), "dtotal": np.zeros((n, N, N)), "dtotal_sorb": np.zeros((n, N, N))}
    o = abi.ReactionBlocksOut(*[out[k].ctypes.data for k in ("res", "jac", "total", "dtotal", "total_sorb",
                                                             "dtotal_sorb")])
    s = cells.struct()
    if lib().pfo_reaction_blocks(C.byref(net_struct), C.byref(opt), C.byref(s), C.byref(o)):
        raise RuntimeError("pfo_reaction_blocks failed")
    return out


def update_mineral_properties(net_struct, cells, mu):
    """Restated porosity / mineral surface-area update on a host CellBatch."""
    s = cells.struct()
    return lib().pfo_update_mineral_properties(C.byref(net_struct), C.byref(s), C.byref(mu))


def equilibrate_constraints(net_struct, opt, cells, types, values, minerals=None, max_iterations=0, nthreads=None,
                            gases=None):
    """Restated constraint speciation of every cell of a host CellBatch;
    `values` (N, ncells), `gases` the network's gas_table() for GAS rows.
    Returns the number of failed cells (< 0: invalid rows)."""
    from pflotran_gb300 import abi
    t = np.ascontiguousarray(types, np.int32)
    mn = None if minerals is None else np.ascontiguousarray(minerals, np.int32)
    v = np.ascontiguousarray(values, np.float64)
    con = abi.constraint(t, v.ctypes.data, mn, max_iterations, gases)
    s = cells.struct()
    return lib().pfo_equilibrate_constraints(C.byref(net_struct), C.byref(opt), C.byref(s), C.byref(con),
                                             nthreads or os.cpu_count() or 1)
