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
    l.pfchem_check_specialized.argtypes = [C.POINTER(abi.Network), C.POINTER(abi.Options), C.c_int, C.c_char_p,
                                           C.c_size_t]
    _lib = l
    return l


class ReactionStep:
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
