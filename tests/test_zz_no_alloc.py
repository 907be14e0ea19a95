"""pfchem_react_batch_noalloc against pfchem_react_batch, through the C ABI.

The allocation-free entry point serves callers that may not allocate device
memory (their device memory comes from their own pool, or cudaMalloc's
device synchronisation is not acceptable inside their time step).  Its only
scratch is a static device array shared by all calls, so this test calls it
twice in a row on fresh copies of the same cells: the second call must not
see state left by the first.  Both calls must match the context-based entry
point to the parity tolerance (1e-10 scaled relative error).
"""
import ctypes as C

import numpy as np
import pytest

from pflotran_gb300 import abi, workloads
from pflotran_gb300.lib import ReactionStep, load

from helpers import compare

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _noalloc(lib):
    f = lib.pfchem_react_batch_noalloc
    f.argtypes = [C.POINTER(abi.Network), C.POINTER(abi.Options), C.c_double, C.POINTER(abi.Cells), C.c_void_p,
                  C.POINTER(abi.Stats), C.c_char_p, C.c_size_t]
    f.restype = C.c_int
    return f


@pytest.mark.parametrize("kind", ["calcite", "synthetic"])
def test_noalloc_matches_react_batch_on_two_calls(kind):
    import torch
    if kind == "calcite":
        net, opt, cells, dt = workloads.calcite_cells(3000, seed=21, temperature_dependent=True)
    else:
        net, opt, cells, dt = workloads.synthetic_cells(3000, seed=22)
    cells.sec_molal = np.zeros(max(net.Nc, 1) * cells.ncells)
    step = ReactionStep(net, opt)
    ref_d = cells.to_device()
    step.react(ref_d, dt)
    ref = ref_d.to_host()
    fn = _noalloc(load())
    ns = net.as_struct()
    for call in range(2):
        d = cells.to_device()
        s = d.struct()
        st = abi.Stats()
        err = C.create_string_buffer(512)
        r = fn(C.byref(ns), C.byref(opt), dt, C.byref(s), None, C.byref(st), err, 512)
        assert r >= 0, err.value.decode()
        torch.cuda.synchronize()
        got = d.to_host()
        ok = ref.status == 0
        assert np.array_equal(got.status, ref.status)
        errs = compare(net, got, ref, mask=ok)
        assert all(v <= TOL for v in errs.values()), (call, errs)
        assert st.ncells == cells.ncells
        assert st.sum_iterations == int(got.iterations.sum())
        assert st.max_iterations == int(got.iterations.max())
        assert st.nonconverged == int((got.status != 0).sum()) == r


def test_noalloc_rejects_host_pointers():
    net, opt, cells, dt = workloads.calcite_cells(10, seed=23)
    fn = _noalloc(load())
    err = C.create_string_buffer(256)
    r = fn(C.byref(net.as_struct()), C.byref(opt), dt, C.byref(cells.struct()), None, None, err, 256)
    assert r == -1 and b"device pointers" in err.value
