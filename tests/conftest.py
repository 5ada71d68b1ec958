import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(GOLDEN, "se_small.npz"), allow_pickle=True))


@pytest.fixture(scope="session")
def kernels_golden():
    return dict(np.load(os.path.join(GOLDEN, "kernels.npz"), allow_pickle=True))


def split_genome(g):
    lens = g["chrom_lens"]
    out, o = [], 0
    for L in lens:
        out.append(np.ascontiguousarray(g["genome"][o:o + L]))
        o += L
    return out


@pytest.fixture(scope="session")
def golden_genome(golden):
    return split_genome(golden)


@pytest.fixture(scope="session")
def oracle_index(golden_genome):
    from oracle.oracle import OracleIndex
    return OracleIndex.build(golden_genome, readlen=100)


@pytest.fixture(scope="session")
def product_index(golden_genome):
    from fame_gb300 import HostIndex
    return HostIndex.build(golden_genome, readlen=100)


@pytest.fixture(scope="session")
def pe_golden():
    return dict(np.load(os.path.join(GOLDEN, "pe_small.npz"), allow_pickle=True))
