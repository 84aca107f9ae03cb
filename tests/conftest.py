import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a GB300 (runs the CUDA library on the device)")


def golden(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def gpu():
    """Both precision builds, initialised on cuda:0.  Fails (never skips) when
    the library or the device is missing: a GPU test must not pass silently."""
    import libmat_gb300 as mg
    libs = {p: mg.load(p) for p in ("f32", "f64")}
    for L in libs.values():
        rc = L.c.matgb_init(0)
        if rc != 0:
            raise RuntimeError("matgb_init failed: %s" % L.c.matgb_last_error())
    return libs
