"""CPU-side checks of the C ABI boundary (no compute calls: no GPU here)."""
import ctypes as C
import os
import re

import pytest

from quantumlab_gb300 import quest as QB

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    names = set()
    for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b([A-Za-z_]\w*)\s*\(([^;{]*)\)\s*;", src, re.M):
        name = m.group(1)
        if m.group(0).lstrip().startswith("typedef") or name in ("void",):
            continue
        names.add(name)
    return names


@pytest.fixture(scope="module")
def product_lib():
    import quantumlab_gb300 as qg
    path = qg.build()
    # load without touching the GPU: symbol lookup only
    return C.CDLL(path, mode=C.RTLD_LOCAL)


def test_every_declared_symbol_is_exported(product_lib):
    for header in ("QuEST.h", "quest_gb300.h"):
        if not os.path.exists(os.path.join(ROOT, "include", header)):
            continue
        names = declared_functions(header)
        assert len(names) >= 4, header
        missing = [n for n in sorted(names) if not hasattr(product_lib, n)]
        assert not missing, f"{header}: not exported: {missing}"


def test_quest_header_covers_the_hot_path():
    names = declared_functions("QuEST.h")
    for fn in ["createQureg", "createDensityQureg", "destroyQureg", "compactUnitary", "unitary",
               "controlledUnitary", "multiControlledUnitary", "controlledNot", "controlledPhaseShift",
               "multiRotatePauli", "mixDephasing", "mixDepolarising", "mixDamping", "calcProbOfOutcome",
               "calcTotalProb", "calcInnerProduct", "calcExpecPauliSum", "initStateFromAmps"]:
        assert fn in names, fn


def test_struct_layouts_match_the_reference_abi():
    # QuEST.h (reference) layouts on LP64: Qureg = 3 ints, 2 long long, 2 ints,
    # 3 ComplexArray, 2 pointers, 1 pointer
    assert C.sizeof(QB.Qureg) == 4 * 3 + 4 + 8 * 2 + 4 * 2 + 16 * 3 + 8 * 2 + 8
    assert QB.Qureg.numAmpsPerChunk.offset == 16
    assert QB.Qureg.stateVec.offset == 40
    assert QB.Qureg.deviceStateVec.offset == 72
    assert C.sizeof(QB.ComplexMatrix2) == 64
    assert C.sizeof(QB.ComplexMatrix4) == 256
    assert C.sizeof(QB.QuESTEnv) == 4 + 4 + 8 + 4 + 4


def test_oracle_exports_the_same_api(oracle):
    names = declared_functions("QuEST.h")
    missing = [n for n in sorted(names) if not oracle.has(n)]
    assert not missing, missing


def test_error_hook_is_overridable(product_lib):
    # the default handler is a weak symbol and a function-pointer hook exists
    assert hasattr(product_lib, "invalidQuESTInputError")
    C.c_void_p.in_dll(product_lib, "__other_input_error")
