"""Shared test setup: import paths, the `gpu` marker, golden-fixture loading."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "td-bem_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    """Single-region full-march cases (two-region ones are named mrt_*, row-block
    ones rows_*)."""
    return sorted(n for n in (os.path.basename(p)[:-4]
                              for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
                  if not n.startswith(("mrt_", "rows_")))


def mrt_golden_cases():
    return sorted(os.path.basename(p)[:-4]
                  for p in glob.glob(os.path.join(GOLDEN, "mrt_*.npz")))


def load_mrt_golden(name):
    """The fixture and the two region models."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    from tdbem import inputfile
    return z, inputfile.parse(str(z["input_text_1"])), inputfile.parse(str(z["input_text_2"]))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    from tdbem import inputfile
    return z, inputfile.parse(str(z["input_text"]))


def rel_max(a, b):
    """max |a - b| / max |b|  (0 when both are zero)."""
    den = np.abs(b).max()
    num = np.abs(a - b).max()
    return 0.0 if num == 0 else num / max(den, 1e-300)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
