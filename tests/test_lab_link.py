"""QuantumLab links against libquest_gb300.so with no source change.

A C++ translation unit written the way QuantumLab's sources use QuEST
(QuEST_precision.h included by name first, as Code/QuantumLab/Base/QLSetup.h:23
does, then QuEST.h) takes the address of every QuEST function the lab calls
and reads the Qureg fields it reads; it is compiled with g++ and linked
against the built product library, then run (it calls nothing on the GPU).
The function list is every QuEST API name that appears in the lab's sources:
the gate dispatch of Circuit/QLGate.cpp:652-804, the simulators of
Simulator/*.cpp, Circuit/Subroutine/QKMeans.cu and
Circuit/Hamitonian/CHamitonianTerm.cpp.  A C translation unit checks the
C-only matrix helpers with their variable-length-array prototypes.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

LAB_CALLS = [
    "calcFidelity", "calcProbOfAllOutcomes", "calcPurity", "collapseToOutcome", "controlledNot",
    "controlledPauliY", "controlledPhaseFlip", "controlledPhaseShift", "controlledRotateX", "controlledRotateY",
    "controlledRotateZ", "copyStateFromGPU", "copyStateToGPU", "createDensityQureg", "createQuESTEnv",
    "createQureg", "destroyQuESTEnv", "destroyQureg", "hadamard", "measure", "mixDamping", "mixDephasing",
    "mixDepolarising", "mixPauli", "mixTwoQubitDephasing", "mixTwoQubitDepolarising", "pauliX", "pauliY",
    "pauliZ", "phaseShift", "rotateX", "rotateY", "rotateZ", "syncQuESTEnv", "unitary",
]
# the rest of the simulation path the benchmark spec names
HOT_PATH = [
    "compactUnitary", "controlledUnitary", "multiControlledUnitary", "multiStateControlledUnitary",
    "multiRotatePauli", "multiRotateZ", "calcProbOfOutcome", "calcTotalProb", "calcInnerProduct",
    "calcExpecPauliSum", "initStateFromAmps", "initZeroState", "applyTrotterCircuit",
]

LAB_TU = r"""
#include "QuEST_precision.h"
#include "QuEST.h"
#include <cstdio>
#include <cstring>

#if QuEST_PREC == 1
#error "the lab selects FP64 amplitudes (QuEST_PREC 2)"
#endif

typedef void (*fn_t)(void);
static fn_t table[] = {
%(entries)s
};

// the fields the lab's simulators read (QLSimulatorVector.cpp:44-49,
// QLSimulatorDensityMatrix.cpp:39, QKMeans.cu:1207-1211)
static long long touch(Qureg q) {
    qreal* re = q.stateVec.real;
    qreal* im = q.stateVec.imag;
    return (long long)(re != nullptr) + (long long)(im != nullptr) + q.numAmpsTotal + q.isDensityMatrix +
           q.numQubitsRepresented + (long long)sizeof(qreal);
}

int main() {
    Qureg q;
    std::memset(&q, 0, sizeof q);
    int n = 0;
    for (fn_t f : table) n += (f != nullptr);
    std::printf("%%d %%lld %%d\n", n, touch(q), Ceil(10, 4));
    return 0;
}
"""

C_TU = r"""
#include "QuEST.h"
#include <stdio.h>
int main(void) {
    qreal re[2][2] = {{1, 0}, {0, 1}}, im[2][2] = {{0, 0}, {0, 0}};
    qreal* rs[2];
    qreal* is[2];
    ComplexMatrixN m = bindArraysToStackComplexMatrixN(1, re, im, rs, is);
    void (*init)(ComplexMatrixN, qreal[][1 << m.numQubits], qreal[][1 << m.numQubits]) = initComplexMatrixN;
    printf("%d %g %d\n", m.numQubits, m.real[1][1], init != 0);
    return 0;
}
"""


@pytest.fixture(scope="module")
def product_so():
    import quantumlab_gb300 as qg
    return qg.build()


def _compile_and_run(tmp_path, src_name, src, compiler, std, so):
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not available")
    src_path = tmp_path / src_name
    src_path.write_text(src)
    exe = tmp_path / (src_name + ".out")
    libdir = os.path.dirname(so)
    cmd = [compiler, std, "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src_path), "-o", str(exe),
           "-L" + libdir, "-l:" + os.path.basename(so), "-Wl,-rpath," + libdir]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stderr
    return run.stdout.split()


def test_lab_translation_unit_links(tmp_path, product_so):
    names = LAB_CALLS + HOT_PATH
    entries = ",\n".join(f"    reinterpret_cast<fn_t>(&{n})" for n in names)
    out = _compile_and_run(tmp_path, "lab_tu.cpp", LAB_TU % {"entries": entries}, "g++", "-std=c++14", product_so)
    assert int(out[0]) == len(names)
    assert int(out[1]) == 8                    # sizeof(qreal) of an empty register
    assert int(out[2]) == 3                    # Ceil(10, 4)


def test_c_only_matrix_helpers_link(tmp_path, product_so):
    out = _compile_and_run(tmp_path, "helpers.c", C_TU, "gcc", "-std=gnu99", product_so)
    assert out == ["1", "1", "1"]


def test_lab_call_list_is_declared():
    """Every function the lab calls is declared in include/QuEST.h."""
    from test_abi import declared_functions
    names = declared_functions("QuEST.h")
    assert not [n for n in LAB_CALLS + HOT_PATH if n not in names]
