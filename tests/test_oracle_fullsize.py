"""The oracle pinned to the reference's own build at the configurations' own
sizes (CPU): the 512 x 256 wind with every term on and hydro only after
100 steps, and one model of each grid size of the 64-model batch (own L_x,
k and alpha) after 20 steps, bit for bit against the digests that
tests/golden/make_golden.py recorded from the reference.  The GPU tests of tests/test_gpu_fullsize.py
then compare the device with the oracle at these sizes."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def _cases():
    return sorted(f[:-5] for f in os.listdir(GOLDEN)
                  if f.endswith(".json") and (f.startswith("wind2d_full_512") or
                                              f.startswith("wind2d_hydro_512") or
                                              f.startswith("wind2d_batch_m")))


@pytest.mark.parametrize("name", _cases())
def test_oracle_matches_reference_at_full_size(built, name):
    from oracle import wind_oracle
    meta = json.load(open(os.path.join(GOLDEN, name + ".json")))
    nr, nt = meta["n"][0], meta["n"][1]
    o = wind_oracle(nr, nt, cooling=meta.get("cooling", 1), line_force=meta.get("line_force", 1),
                    l_star=meta["l_star"], krad=meta["krad"], alpharad=meta["alpharad"])
    assert _digest(o.active()) == meta["ic_sha256"]
    o.run(meta["steps"])
    a = o.active()
    assert _digest(a) == meta["final_sha256"], name
    assert np.allclose(a.reshape(6, -1).sum(axis=1), meta["final_sums"], rtol=0, atol=0)
    t, dt, step = o.time()
    assert step == meta["steps"]
    assert "%e" % t == meta["t"][1]
