"""Builds the in-tree CUDA libraries for sm_103a with nvcc: libpfchem.so
(the chemistry library), libpfchem_probe.so (the FP64 peak probe) and
libpfchem_transport.so (the time-stepped run's upwind transport).

Translation units compiled in parallel, then linked; output in
pflotran_gb300/_build/.  Re-running skips the build when no source changed.
"""
import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpfchem.so")
PROBE = os.path.join(OUT, "libpfchem_probe.so")
SOURCES = ["pfchem_newton.cu", "pfchem_api.cu", "pfchem_noalloc.cu", "pfchem_codegen.cu", "pfchem_mlp.cu",
           "pfchem_coop.cu", "pfchem_umma.cu"]
PROBE_SOURCES = ["fp64_peak.cu"]
TRANSPORT = os.path.join(OUT, "libpfchem_transport.so")
TRANSPORT_SOURCES = ["transport_upwind.cu"]
HEADERS = ["pfchem_device.cuh", os.path.join("..", "..", "include", "pfchem.h")]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _cuda_home():
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _digest():
    h = hashlib.sha256()
    for f in SOURCES + PROBE_SOURCES + TRANSPORT_SOURCES + HEADERS:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "stamp")
    dig = _digest()
    if (not force and os.path.exists(LIB) and os.path.exists(PROBE) and os.path.exists(TRANSPORT)
            and os.path.exists(stamp)
            and open(stamp).read() == dig):
        return LIB
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    all_src = SOURCES + PROBE_SOURCES + TRANSPORT_SOURCES
    with ThreadPoolExecutor(len(all_src)) as ex:
        objs = list(ex.map(compile_one, all_src))
    a, b = len(SOURCES), len(SOURCES) + len(PROBE_SOURCES)
    for target, o in ((LIB, objs[:a]), (PROBE, objs[a:b]), (TRANSPORT, objs[b:])):
        tmp = target + ".tmp"
        cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + o
        if target == LIB:
            cmd += ["-L" + os.path.join(_cuda_home(), "lib64"),
                    "-lnvrtc"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, target)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
