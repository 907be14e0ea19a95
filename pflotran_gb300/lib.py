"""Loader for the in-tree CUDA library and the host-side mirror of PFLOTRAN's
operator-split reaction interface.

`ReactionStep` plays the role of the reaction object plus the RTReact driver
(src/pflotran/reactive_transport.F90:1605-1806): it is configured once with
the network tables and options (reaction_type and the CHEMISTRY options of
reaction.F90:755-857) and then advances batches of cells by one reaction step
(RReact per cell, reaction.F90:3322-3511) on the GPU.  Errors the reference
reports through printErrMsg (bad tables, unsupported options) raise
PfchemError; per-cell non-convergence is reported as per-cell status codes
(the reference would stop the run).

There is no CPU path: if the CUDA library or a GPU is missing, construction
fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpfchem.so")
_HEADER = os.path.join(os.path.dirname(_HERE), "include", "pfchem.h")
_lib = None


class PfchemError(RuntimeError):
    pass


def header_functions():
    """Function names declared in include/pfchem.h."""
    txt = open(_HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pfchem_\w+)\s*\(", txt)))


def load(build_if_missing=True):
    """Loads libpfchem.so (building it with nvcc when missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        if not build_if_missing:
            raise PfchemError(f"CUDA library not built: {_LIB_PATH}")
        from .build import build
        build()
    l = C.CDLL(_LIB_PATH)
    vp = C.c_void_p
    l.pfchem_create.argtypes = [C.POINTER(vp), C.c_int]
    l.pfchem_destroy.argtypes = [vp]
    l.pfchem_destroy.restype = None
    l.pfchem_last_error.argtypes = [vp]
    l.pfchem_last_error.restype = C.c_char_p
    l.pfchem_set_network.argtypes = [vp, C.POINTER(abi.Network), C.POINTER(abi.Options)]
    l.pfchem_react_batch.argtypes = [vp, C.c_double, C.POINTER(abi.Cells)]
    l.pfchem_react_batch_interleaved.argtypes = [vp, C.c_double, C.c_int32, vp, C.POINTER(abi.Cells)]
    l.pfchem_update_kinetic_state.argtypes = [vp, C.c_double, C.POINTER(abi.Cells)]
    l.pfchem_last_stats.argtypes = [vp, C.POINTER(abi.Stats)]
    l.pfchem_get_launch.argtypes = [vp, C.POINTER(abi.Launch)]
    l.pfchem_set_launch.argtypes = [vp, C.POINTER(abi.Launch)]
    l.pfchem_autotune.argtypes = [vp, C.c_double, C.POINTER(abi.Cells)]
    l.pfchem_reaction_blocks.argtypes = [vp, C.POINTER(abi.Cells), C.POINTER(abi.ReactionBlocksOut)]
    l.pfchem_update_mineral_properties.argtypes = [vp, C.POINTER(abi.Cells), C.POINTER(abi.MineralUpdate)]
    l.pfchem_equilibrate_constraints.argtypes = [vp, C.POINTER(abi.Cells), C.POINTER(abi.Constraint)]
    l.pfchem_reserve.argtypes = [vp, C.c_int64]
    l.pfchem_react_batch_async.argtypes = [vp, C.c_double, C.POINTER(abi.Cells), vp]
    l.pfchem_async_stats.argtypes = [vp, C.POINTER(abi.Stats)]
    l.pfchem_check_specialized.argtypes = [C.POINTER(abi.Network), C.POINTER(abi.Options), C.c_int, C.c_char_p,
                                           C.c_size_t]
    _lib = l
    return l


class SurrogateConfig(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("weight_decay", C.c_float),
                ("seed", C.c_uint64)]


class SurrogateReport(C.Structure):
    _fields_ = [("samples", C.c_int64), ("steps", C.c_int64), ("first_loss", C.c_float),
                ("final_loss", C.c_float), ("train_ms", C.c_double)]


def _surrogate_bind(l):
    vp = C.c_void_p
    l.pfchem_surrogate_features.argtypes = [vp, C.POINTER(abi.Cells), vp]
    l.pfchem_surrogate_fit.argtypes = [vp, vp, vp, C.c_int64, C.POINTER(SurrogateConfig),
                                       C.POINTER(SurrogateReport)]
    l.pfchem_surrogate_enable.argtypes = [vp, C.c_int]
    l.pfchem_surrogate_predict_layers.argtypes = [vp, C.POINTER(abi.Cells), vp]
    l.pfchem_surrogate_predict.argtypes = [vp, C.POINTER(abi.Cells), vp]
    l.pfchem_surrogate_gradients.argtypes = [vp, vp, vp, C.c_int64, vp, vp]
    l.pfchem_surrogate_gradients.restype = C.c_int64
    l.pfchem_surrogate_params.argtypes = [vp, vp, C.c_int]
    l.pfchem_surrogate_params.restype = C.c_int64
    l.pfchem_surrogate_normalization.argtypes = [vp, vp, vp, vp, vp, C.c_int]
    l.pfchem_surrogate_backend.argtypes = [vp, C.c_int]


class WarmStartMixin:
    """Learned warm start on a ReactionStep (all tensors on the device)."""

    def surrogate_features(self, cells):
        import torch
        _surrogate_bind(self._lib)
        X = torch.empty((cells.ncells, 16), dtype=torch.float32, device="cuda")
        s = cells.struct()
        self._check(self._lib.pfchem_surrogate_features(self._ctx, C.byref(s), C.c_void_p(X.data_ptr())),
                    "pfchem_surrogate_features")
        return X

    def surrogate_fit(self, X, molal_soa, epochs=8, batch=8192, lr=2e-3, weight_decay=1e-4, seed=7):
        _surrogate_bind(self._lib)
        M = X.shape[0]
        cfg = SurrogateConfig(epochs, batch, lr, weight_decay, seed)
        rep = SurrogateReport()
        self._check(self._lib.pfchem_surrogate_fit(self._ctx, C.c_void_p(X.data_ptr()),
                                                   C.c_void_p(molal_soa.data_ptr()), M, C.byref(cfg),
                                                   C.byref(rep)), "pfchem_surrogate_fit")
        return rep

    def surrogate_predict(self, cells):
        import torch
        _surrogate_bind(self._lib)
        g = torch.empty(self.network.N * cells.ncells, dtype=torch.float64, device="cuda")
        s = cells.struct()
        self._check(self._lib.pfchem_surrogate_predict(self._ctx, C.byref(s), C.c_void_p(g.data_ptr())),
                    "pfchem_surrogate_predict")
        return g

    def surrogate_predict_layers(self, cells):
        """The layer-by-layer (GEMM per layer) prediction, to check the fused kernel."""
        import torch
        _surrogate_bind(self._lib)
        g = torch.empty(self.network.N * cells.ncells, dtype=torch.float64, device="cuda")
        s = cells.struct()
        self._check(self._lib.pfchem_surrogate_predict_layers(self._ctx, C.byref(s), C.c_void_p(g.data_ptr())),
                    "pfchem_surrogate_predict_layers")
        return g

    def surrogate_backend(self, backend):
        """Tensor-core path of the dense layers: abi.MLP_MMA_SYNC or abi.MLP_TCGEN05."""
        _surrogate_bind(self._lib)
        self._check(self._lib.pfchem_surrogate_backend(self._ctx, int(backend)), "pfchem_surrogate_backend")

    def surrogate_enable(self, on=True):
        _surrogate_bind(self._lib)
        self._check(self._lib.pfchem_surrogate_enable(self._ctx, int(on)), "pfchem_surrogate_enable")

    def surrogate_gradients(self, X, molal_soa):
        import numpy as np
        _surrogate_bind(self._lib)
        n = self._lib.pfchem_surrogate_params(self._ctx, None, 0)
        g = np.zeros(n, np.float32)
        loss = np.zeros(1, np.float32)
        r = self._lib.pfchem_surrogate_gradients(self._ctx, C.c_void_p(X.data_ptr()),
                                                 C.c_void_p(molal_soa.data_ptr()), X.shape[0],
                                                 g.ctypes.data, loss.ctypes.data)
        self._check(r, "pfchem_surrogate_gradients")
        return g, float(loss[0])

    def surrogate_params(self, values=None):
        import numpy as np
        _surrogate_bind(self._lib)
        n = self._lib.pfchem_surrogate_params(self._ctx, None, 0)
        self._check(n, "pfchem_surrogate_params")
        if values is None:
            out = np.zeros(n, np.float32)
            self._lib.pfchem_surrogate_params(self._ctx, out.ctypes.data, 0)
            return out
        v = np.ascontiguousarray(values, np.float32)
        assert v.size == n
        self._check(self._lib.pfchem_surrogate_params(self._ctx, v.ctypes.data, 1), "pfchem_surrogate_params")

    def surrogate_normalization(self, values=None):
        import numpy as np
        _surrogate_bind(self._lib)
        N = self.network.N
        if values is None:
            fm, fs, tm, ts = (np.zeros(16, np.float32), np.zeros(16, np.float32), np.zeros(N, np.float32),
                              np.zeros(N, np.float32))
            self._check(self._lib.pfchem_surrogate_normalization(self._ctx, fm.ctypes.data, fs.ctypes.data,
                                                                 tm.ctypes.data, ts.ctypes.data, 0), "norm")
            return fm, fs, tm, ts
        fm, fs, tm, ts = [np.ascontiguousarray(a, np.float32) for a in values]
        self._check(self._lib.pfchem_surrogate_normalization(self._ctx, fm.ctypes.data, fs.ctypes.data,
                                                             tm.ctypes.data, ts.ctypes.data, 1), "norm")



class ReactionStep(WarmStartMixin):
    """Batched operator-split reaction step on one GPU."""

    def __init__(self, network, options=None, device=0):
        import torch
        if not torch.cuda.is_available():
            raise PfchemError("no CUDA device: the reaction step runs only on the GPU")
        self._lib = load()
        self._ctx = C.c_void_p()
        r = self._lib.pfchem_create(C.byref(self._ctx), device)
        if r != 0:
            raise PfchemError(f"pfchem_create failed ({r})")
        self.network = network
        self.options = options
        self._net_struct = network.as_struct() if hasattr(network, "as_struct") else network
        self._check(self._lib.pfchem_set_network(self._ctx, C.byref(self._net_struct), C.byref(options)),
                    "pfchem_set_network")

    def set_options(self, options):
        """New CHEMISTRY options for the same network (the trained warm
        start, if any, is kept)."""
        self.options = options
        self._check(self._lib.pfchem_set_network(self._ctx, C.byref(self._net_struct), C.byref(options)),
                    "pfchem_set_network")

    def _check(self, r, what):
        if r < 0:
            msg = self._lib.pfchem_last_error(self._ctx).decode()
            raise PfchemError(f"{what} failed ({r}): {msg}")
        return r

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.pfchem_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def react(self, cells, dt):
        """RTReact over `cells` (a CellBatch on the host or the device).
        Returns the number of cells whose status is not CONVERGED."""
        s = cells.struct()
        return self._check(self._lib.pfchem_react_batch(self._ctx, dt, C.byref(s)), "pfchem_react_batch")

    def react_interleaved(self, tran_xx, ncomp, cells, dt):
        """RTReact on its own interleaved tran_xx layout (ncomp per cell)."""
        s = cells.struct()
        ptr = tran_xx.data_ptr() if hasattr(tran_xx, "data_ptr") else tran_xx.ctypes.data
        return self._check(self._lib.pfchem_react_batch_interleaved(self._ctx, dt, ncomp, C.c_void_p(ptr),
                                                                    C.byref(s)),
                           "pfchem_react_batch_interleaved")

    def reserve(self, ncells):
        """Sizes the device buffers so that react_async allocates nothing."""
        self._check(self._lib.pfchem_reserve(self._ctx, int(ncells)), "pfchem_reserve")

    def react_async(self, cells, dt, stream):
        """Enqueues one reaction step of device-resident `cells` on `stream`
        (a torch.cuda.Stream or a raw cudaStream_t handle) without waiting;
        capturable into a CUDA graph.  The CellBatch struct is kept alive on
        the object, since a captured graph holds the pointers it names."""
        self._async_struct = cells.struct()
        h = getattr(stream, "cuda_stream", stream)
        return self._check(self._lib.pfchem_react_batch_async(self._ctx, dt, C.byref(self._async_struct),
                                                              C.c_void_p(h)), "pfchem_react_batch_async")

    def async_stats(self):
        """Statistics of the last completed react_async step (synchronise its stream first)."""
        st = abi.Stats()
        self._check(self._lib.pfchem_async_stats(self._ctx, C.byref(st)), "pfchem_async_stats")
        return st

    def equilibrate_constraints(self, cells, types, values, minerals=None, max_iterations=0):
        """Constraint speciation of every cell of a device batch: `types`
        and 1-based `minerals` (the constraint_spec_id: the kinetic mineral
        of a MINERAL row, the network's passive gas of a GAS row) per
        component, `values` a device tensor (N, ncells).  Returns the number
        of cells that did not converge."""
        import numpy as np
        t = np.ascontiguousarray(types, np.int32)
        mn = None if minerals is None else np.ascontiguousarray(minerals, np.int32)
        gases = self.network.gas_table() if self.network.gases else None
        con = abi.constraint(t, values.data_ptr(), mn, max_iterations, gases)
        s = cells.struct()
        return self._check(self._lib.pfchem_equilibrate_constraints(self._ctx, C.byref(s), C.byref(con)),
                           "pfchem_equilibrate_constraints")

    def reaction_blocks(self, cells):
        """Global-implicit per-cell blocks at the cells' current state (device
        batch): dict of device tensors res (N, ncells), jac / dtotal /
        dtotal_sorb (ncells, N, N) with [c, j, i] = d(.)_i/dm_j, total and
        total_sorb (N, ncells)."""
        import torch
        N, n = self.network.N, cells.ncells
        out = {"res": torch.empty((N, n), dtype=torch.float64, device="cuda"),
               "total": torch.empty((N, n), dtype=torch.float64, device="cuda"),
               "total_sorb": torch.empty((N, n), dtype=torch.float64, device="cuda")}
        for k in ("jac", "dtotal", "dtotal_sorb"):
            out[k] = torch.empty((n, N, N), dtype=torch.float64, device="cuda")
        o = abi.ReactionBlocksOut(*[out[k].data_ptr() for k in ("res", "jac", "total", "dtotal", "total_sorb",
                                                                  "dtotal_sorb")])
        s = cells.struct()
        self._check(self._lib.pfchem_reaction_blocks(self._ctx, C.byref(s), C.byref(o)), "pfchem_reaction_blocks")
        return out

    def update_mineral_properties(self, cells, mu):
        """Porosity and mineral surface area from the volume fractions
        (device batch; `mu` an abi.MineralUpdate over device arrays)."""
        s = cells.struct()
        return self._check(self._lib.pfchem_update_mineral_properties(self._ctx, C.byref(s), C.byref(mu)),
                           "pfchem_update_mineral_properties")

    def update_kinetic_state(self, cells, dt):
        """RTUpdateKineticState (device batches only)."""
        s = cells.struct()
        return self._check(self._lib.pfchem_update_kinetic_state(self._ctx, dt, C.byref(s)),
                           "pfchem_update_kinetic_state")

    def stats(self):
        st = abi.Stats()
        self._lib.pfchem_last_stats(self._ctx, C.byref(st))
        return st

    def launch(self):
        l = abi.Launch()
        self._lib.pfchem_get_launch(self._ctx, C.byref(l))
        return l

    def set_launch(self, block_threads, blocks_per_sm, refill_min_idle, variant=abi.KERNEL_SPECIALIZED):
        l = abi.Launch(block_threads, blocks_per_sm, refill_min_idle, variant)
        self._check(self._lib.pfchem_set_launch(self._ctx, C.byref(l)), "pfchem_set_launch")

    def autotune(self, cells, dt):
        s = cells.struct()
        self._check(self._lib.pfchem_autotune(self._ctx, dt, C.byref(s)), "pfchem_autotune")
        return self.launch()
