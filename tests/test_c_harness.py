"""A C caller of the library (tests/rtreact_harness.c) that fills the network
tables in reaction_type's layout and calls the batched step on RTReact's
interleaved tran_xx, as the Fortran driver would.  On the CPU: the tables
compile into the network-specialized kernel (NVRTC, no GPU), the harness
fails cleanly without a GPU, and the same tables and arrays run through the
oracle give bit for bit what the Python-built network gives.  On the GPU:
parity of the harness's step with the oracle."""
import os
import subprocess

import numpy as np
import pytest

from pflotran_gb300 import workloads

from helpers import compare

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(ROOT, "pflotran_gb300", "_build")
ORACLE_LIBDIR = os.path.join(ROOT, "oracle", "_build")
N = 3


@pytest.fixture(scope="module")
def harness(tmp_path_factory, oracle):
    from pflotran_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp("harness") / "rtreact_harness")
    cuda_lib = os.path.join(build._cuda_home(), "lib64")  # libnvrtc, which libpfchem links
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-DWITH_ORACLE", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "rtreact_harness.c"), "-o", exe,
           "-L", LIBDIR, "-lpfchem", "-L", ORACLE_LIBDIR, "-lpfchem_oracle",
           f"-Wl,-rpath,{LIBDIR}", f"-Wl,-rpath,{ORACLE_LIBDIR}", f"-Wl,-rpath,{cuda_lib}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _write_input(path, cells, dt):
    n = cells.ncells
    with open(path, "wb") as f:
        f.write(np.int64(n).tobytes())
        f.write(np.float64(dt).tobytes())
        for a in (cells.temperature, cells.saturation, cells.den_kg, cells.porosity, cells.volume, cells.total,
                  cells.pri_molal, cells.ionic_strength, cells.mnrl_volfrac, cells.mnrl_area):
            f.write(np.ascontiguousarray(a, np.float64).tobytes())


def _read_output(path, n):
    raw = open(path, "rb").read()
    rc = int(np.frombuffer(raw[:4], np.int32)[0])
    off = 4
    out = {}
    for name, count, dtype in (("tran_xx", N * n, np.float64), ("pri_molal", N * n, np.float64),
                               ("total_out", N * n, np.float64), ("mnrl_rate", n, np.float64),
                               ("mnrl_volfrac", n, np.float64), ("ionic_strength", n, np.float64),
                               ("iterations", n, np.int32), ("status", n, np.int32)):
        size = count * np.dtype(dtype).itemsize
        out[name] = np.frombuffer(raw[off:off + size], dtype).copy()
        off += size
    assert off == len(raw)
    return rc, out


def _reference(oracle, n, seed):
    net, opt, cells, dt = workloads.calcite_cells(n, seed=seed)
    ref = cells.copy()
    ref.sec_molal = np.zeros(net.Nc * n)
    oracle.react(net.as_struct(), opt, dt, ref, 0, 4)
    return net, cells, dt, ref


def test_harness_tables_compile_into_the_specialized_kernel(harness):
    r = subprocess.run([harness, "check"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "check ok" in r.stdout


def test_harness_tables_through_the_oracle_match_the_python_network(harness, oracle, tmp_path):
    """The harness's C tables, options and arrays, run through the oracle,
    give bit for bit the oracle's result on the Python-built network."""
    net, cells, dt, ref = _reference(oracle, 512, seed=5)
    _write_input(tmp_path / "in.bin", cells, dt)
    r = subprocess.run([harness, "oracle", str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rc, out = _read_output(tmp_path / "out.bin", cells.ncells)
    assert rc == 0
    n = cells.ncells
    assert np.array_equal(out["pri_molal"], ref.pri_molal)
    # tran_xx holds the free-ion molalities, cell-major, as after reactive_transport.F90:1711
    assert np.array_equal(out["tran_xx"], ref.pri_molal.reshape(N, n).T.ravel())
    for f in ("total_out", "mnrl_rate", "mnrl_volfrac", "ionic_strength"):
        assert np.array_equal(out[f], getattr(ref, f)), f
    assert np.array_equal(out["iterations"], ref.iterations) and np.array_equal(out["status"], ref.status)


def test_harness_fails_cleanly_without_a_gpu(harness, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    net, opt, cells, dt = workloads.calcite_cells(8, seed=1)
    _write_input(tmp_path / "in.bin", cells, dt)
    r = subprocess.run([harness, "run", str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "pfchem_create" in r.stderr


@pytest.mark.gpu
def test_harness_step_on_the_gpu_matches_the_oracle(harness, oracle, tmp_path):
    net, cells, dt, ref = _reference(oracle, 4096, seed=6)
    _write_input(tmp_path / "in.bin", cells, dt)
    r = subprocess.run([harness, "run", str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rc, out = _read_output(tmp_path / "out.bin", cells.ncells)
    assert rc == 0
    gpu = ref.copy()
    for f in ("pri_molal", "total_out", "mnrl_rate", "mnrl_volfrac", "ionic_strength", "iterations", "status"):
        setattr(gpu, f, out[f])
    gpu.sec_molal = None
    n = cells.ncells
    assert np.array_equal(out["tran_xx"], out["pri_molal"].reshape(N, n).T.ravel())
    errs = compare(net, gpu, ref)
    assert all(v <= 1e-10 for v in errs.values()), errs
