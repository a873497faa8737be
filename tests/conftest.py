"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libquest_oracle.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure), built on demand from oracle/."""
    from quantumlab_gb300.quest import QuESTLibrary
    src = os.path.join(ROOT, "oracle", "quest_oracle.c")
    if not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return QuESTLibrary(ORACLE_LIB)


@pytest.fixture(scope="session")
def gpulib():
    """The product library on cuda:0 (built in-tree; no fallback)."""
    import quantumlab_gb300 as qg
    qg.build()
    return qg.load()


@pytest.fixture(scope="session")
def golden():
    import gzip
    import json
    import numpy as np
    here = os.path.join(ROOT, "tests", "golden")
    with gzip.open(os.path.join(here, "api_cases.json.gz"), "rt") as f:
        cases = json.load(f)
    amps = np.load(os.path.join(here, "api_amps.npz"))
    circ = np.load(os.path.join(here, "circuits.npz"))
    return cases, amps, circ
