import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pluto-sirocco_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


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
