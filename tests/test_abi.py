"""The C ABI: every function declared in include/pfchem.h is exported by the
built library, and the ctypes mirror has the C compiler's struct layout."""
import ctypes as C
import os
import subprocess

import pytest

from pflotran_gb300 import abi
from pflotran_gb300.build import build
from pflotran_gb300.lib import header_functions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_builds_and_exports_header_symbols():
    lib_path = build()
    lib = C.CDLL(lib_path)
    names = header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n


@pytest.mark.parametrize("name,cls", [("pfchem_network", abi.Network), ("pfchem_options", abi.Options),
                                      ("pfchem_cells", abi.Cells), ("pfchem_stats", abi.Stats),
                                      ("pfchem_launch", abi.Launch), ("pfchem_constraint", abi.Constraint),
                                      ("pfchem_mineral_update", abi.MineralUpdate),
                                      ("pfchem_reaction_blocks_out", abi.ReactionBlocksOut)])
def test_struct_layout_matches_header(tmp_path, name, cls):
    fields = [f[0] for f in cls._fields_]
    src = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/pfchem.h"', "int main(void){",
           f'printf("%zu\\n", sizeof({name}));']
    for f in fields:
        src.append(f'printf("%zu\\n", offsetof({name}, {f}));')
    src.append("return 0;}")
    c = tmp_path / "probe.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-o", str(exe), str(c)])
    vals = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert vals[0] == C.sizeof(cls)
    for f, off in zip(fields, vals[1:]):
        assert getattr(cls, f).offset == off, f


def test_product_path_has_no_oracle_dependency():
    """The library sources and the package never load or call the oracle."""
    pkg = os.path.join(ROOT, "pflotran_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dirpath, fn)).read()
                for bad in ("import oracle", "from oracle", "pfo_", "libpfchem_oracle"):
                    assert bad not in txt, (fn, bad)
