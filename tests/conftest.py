import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
CASE_NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                    if not p.endswith(("luts.npz", "pils_ops.npz")))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: full-size configuration")


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def frlib():
    from fastrecon_gb300 import build, capi
    build.build()
    return capi.load()


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    p = d["params"]
    d.update(dim=int(p[0]), spokes=int(p[1]), readout=int(p[2]), coils=int(p[3]), recon=int(p[4]),
             os=float(p[5]), W=float(p[6]), L=int(p[7]))
    d["G"] = int(np.float32(d["recon"]) * np.float32(d["os"]))
    d["name"] = name
    return d


@pytest.fixture(params=CASE_NAMES)
def case(request):
    return load_case(request.param)


def rel_l2(a, b):
    a = np.asarray(a).astype(np.complex128).ravel()
    b = np.asarray(b).astype(np.complex128).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)
