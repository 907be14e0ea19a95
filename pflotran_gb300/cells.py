"""Per-cell structure-of-arrays batches for the C ABI.

A `CellBatch` holds every per-cell field of `pfchem_cells` as a numpy array
(host) or a torch tensor (device) with the layout field[i, cell] -> flat
index i * ncells + cell.  `struct()` returns the ctypes `pfchem_cells` that
points at the arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi

_F64 = ("temperature", "saturation", "den_kg", "porosity", "volume", "soil_particle_density",
        "total", "pri_molal", "ionic_strength", "ln_act_h2o", "mnrl_volfrac", "mnrl_area",
        "total_sorb_eq", "eqionx_ref_cation_sorbed_conc", "srfcplxrxn_free_site_conc",
        "total_out", "mnrl_rate", "sec_molal", "alt_guess")
_I32 = ("active", "iterations", "status")


class CellBatch:
    """Named per-cell arrays; missing optional fields are None."""

    FIELDS = _F64 + _I32

    def __init__(self, ncells, **arrays):
        self.ncells = int(ncells)
        for f in self.FIELDS:
            setattr(self, f, arrays.get(f))

    @classmethod
    def allocate(cls, net, ncells, outputs=True, sec_molal=False):
        """Zeroed host batch shaped for `net` (a ReactionNetwork)."""
        n = int(ncells)
        z = lambda k: np.zeros(k * n, dtype=np.float64)
        b = cls(n)
        for f in ("temperature", "saturation", "den_kg", "porosity", "volume",
                  "soil_particle_density", "ionic_strength"):
            setattr(b, f, z(1))
        b.total, b.pri_molal = z(net.N), z(net.N)
        b.mnrl_volfrac, b.mnrl_area = z(max(net.Nm, 1)), z(max(net.Nm, 1))
        if net.Nix + net.Nsr > 0:
            b.total_sorb_eq = z(net.N)
        if net.Nix > 0:
            b.eqionx_ref_cation_sorbed_conc = z(net.Nix)
        if net.Nsr > 0:
            b.srfcplxrxn_free_site_conc = z(net.Nsr)
        if outputs:
            b.total_out, b.mnrl_rate = z(net.N), z(max(net.Nm, 1))
            b.iterations = np.zeros(n, np.int32)
            b.status = np.zeros(n, np.int32)
        if sec_molal:
            b.sec_molal = z(max(net.Nc, 1))
        return b

    def view(self, name, k):
        """field as a (k, ncells) view."""
        a = getattr(self, name)
        return a.reshape(k, self.ncells)

    def copy(self):
        out = CellBatch(self.ncells)
        for f in self.FIELDS:
            a = getattr(self, f)
            if a is not None:
                setattr(out, f, a.clone() if hasattr(a, "clone") else a.copy())
        return out

    def to_device(self, device="cuda"):
        import torch
        out = CellBatch(self.ncells)
        for f in self.FIELDS:
            a = getattr(self, f)
            if a is not None:
                setattr(out, f, torch.from_numpy(np.ascontiguousarray(a)).to(device))
        return out

    def to_host(self):
        out = CellBatch(self.ncells)
        for f in self.FIELDS:
            a = getattr(self, f)
            if a is not None:
                setattr(out, f, a.detach().cpu().numpy() if hasattr(a, "detach") else a.copy())
        return out

    def subset(self, idx, net):
        """Host batch restricted to cells `idx` (numpy index array)."""
        idx = np.asarray(idx)
        out = CellBatch(len(idx))
        for f in self.FIELDS:
            a = getattr(self, f)
            if a is None:
                continue
            k = a.size // self.ncells
            setattr(out, f, np.ascontiguousarray(a.reshape(k, self.ncells)[:, idx]).ravel())
        return out

    def struct(self) -> abi.Cells:
        s = abi.Cells()
        s.ncells = self.ncells
        dev = None
        keep = []
        for f in self.FIELDS:
            a = getattr(self, f)
            if a is None:
                continue
            if hasattr(a, "data_ptr"):
                assert a.is_contiguous()
                dev = a.is_cuda if dev is None else dev
                ptr = a.data_ptr()
            else:
                assert a.flags.c_contiguous
                want = np.int32 if f in _I32 else np.float64
                assert a.dtype == want, (f, a.dtype)
                dev = False if dev is None else dev
                ptr = a.ctypes.data
            keep.append(a)
            setattr(s, f if f != "total_out" else "total_out", C.c_void_p(ptr))
        s.on_device = 1 if dev else 0
        s._keep = keep
        return s
