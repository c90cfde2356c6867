import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ska-spc-tender-benchmarks_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the native kernels")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build(with_ref=False)
    return oracle


@pytest.fixture(scope="session")
def idg():
    import idg_gb300

    idg_gb300.load()
    return idg_gb300


def golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(path):
    z = np.load(path)
    d = {k: z[k] for k in z.files}
    import idg_gb300._lib as L

    d["metadata"] = np.ascontiguousarray(d["metadata"]).view(L.METADATA_DTYPE).reshape(-1)
    d["cfg"] = tuple(int(x) for x in d["cfg"])
    return d


def rel_rms(x, ref):
    x = np.asarray(x, np.complex128)
    ref = np.asarray(ref, np.complex128)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (den if den > 0 else 1.0))


def check_rel(name, x, ref, tol):
    """Relative RMS check that also prints the measured error (visible with pytest -s)."""
    e = rel_rms(x, ref)
    print(f"[parity] {name}: relative RMS {e:.3e} (tolerance {tol:.0e})")
    assert e <= tol, f"{name}: relative RMS {e:.3e} > {tol:.0e}"
    return e
