import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pluto-sirocco_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# Tolerances for the FP64 hydro state against the reference (or the oracle,
# which is bit-identical to it): relative L1 error per variable, and the
# conserved totals.  The device code contracts multiplies and adds into
# FMAs, which the reference's x86-64 build does not; the measured
# differences are 1e-16 to 1e-13.
HYDRO_REL_L1 = 1e-11
CONSERVED_REL = 1e-12


def rel_l1(a, ref):
    """Relative L1 difference per variable (axis 0); variables that are
    identically zero in `ref` are measured against the largest norm."""
    ax = tuple(range(1, np.ndim(a)))
    den = np.abs(ref).sum(axis=ax)
    num = np.abs(np.asarray(a) - ref).sum(axis=ax)
    scale = max(float(den.max()), 1e-300)
    return np.where(den > 0, num / np.maximum(den, 1e-300), num / scale)


def assert_hydro_close(a, ref, what="", tol=HYDRO_REL_L1):
    r = rel_l1(a, ref)
    assert np.all(r <= tol), f"{what}: relative L1 per variable {r} above {tol}"
    return r


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build the C-ABI library and the oracle once per session if missing."""
    import ps_build as pkg_build  # pluto-sirocco_gb300/ps_build.py
    pkg_build.build_lib()
    pkg_build.build_oracle()
    return True


def golden_cases(full_only=False, kind="blast"):
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.json"))):
        meta = json.load(open(f))
        if meta.get("kind", "blast") != kind:
            continue
        npz = f[:-5] + ".npz"
        meta["npz"] = npz if os.path.exists(npz) else None
        if full_only and meta["npz"] is None:
            continue
        out.append(meta)
    return out


def load_golden(meta):
    d = np.load(meta["npz"])
    return d["v0"], d["v1"]


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
