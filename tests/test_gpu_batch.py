"""Batched wind models (ps_batch): several independent line-driven wind
models of uneven grid sizes and parameters advanced together must give
exactly what each model gives when advanced on its own with ps_run, for
every tile shape and after the autotuner has chosen shapes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [
    dict(grid=(64, 32), l_star=1e37, krad=0.2, alpharad=-0.6),
    dict(grid=(96, 48), l_star=3e36, krad=0.35, alpharad=-0.52),
    dict(grid=(128, 64), l_star=6e37, krad=0.12, alpharad=-0.68),
]


def _pairs(cooling):
    # without cooling: the hydro-only wind (no line force either), as the
    # reference's hydro-only configuration
    import psgb
    solo = [psgb.wind_model_solver(s, cooling=cooling, line_force=cooling) for s in SPECS]
    inb = [psgb.wind_model_solver(s, cooling=cooling, line_force=cooling) for s in SPECS]
    return solo, inb


def _check_equal(solo, inb):
    for m, (a, b) in enumerate(zip(solo, inb)):
        va, vb = a.get_state(), b.get_state()
        d = np.abs(va - vb)
        assert np.array_equal(va, vb), f"model {m}: {np.count_nonzero(d)} values differ, max {d.max():.3e}"
        assert a.time()[:2] == b.time()[:2], f"model {m}: t/dt differ"


@pytest.mark.parametrize("cooling", [0, 1])
def test_batch_matches_individual_runs(built, cooling):
    import psgb
    solo, inb = _pairs(cooling)
    batch = psgb.Batch(inb)
    for chunk in (7, 6):   # odd then even chunk: every step graph is used
        flags = 0
        for s in solo:
            flags |= s.run(chunk)
        assert batch.run(chunk) == flags
        _check_equal(solo, inb)
    # the models as parallel groups (here one per model): the same bits
    batch.set_groups(3)
    for chunk in (5, 4):
        for s in solo:
            s.run(chunk)
        batch.run(chunk)
        _check_equal(solo, inb)
    batch.close()


def test_batch_tile_shapes_and_autotune(built):
    import psgb
    solo, inb = _pairs(1)
    batch = psgb.Batch(inb)
    batch.set_shape(1, model=0)
    batch.set_shape(2, model=2)
    assert batch.shape(0) == (16, 16) and batch.shape(1) == (32, 8) and batch.shape(2) == (64, 4)
    for s in solo:
        s.run(5)
    batch.run(5)
    _check_equal(solo, inb)
    t_before = [b.time()[:2] for b in inb]
    batch.autotune(reps=3)
    assert [b.time()[:2] for b in inb] == t_before   # the autotuner leaves the state alone
    for s in solo:
        s.run(6)
    batch.run(6)
    _check_equal(solo, inb)
    for m in range(len(SPECS)):
        assert batch.shape(m) in [(32, 8), (16, 16), (64, 4), (32, 16)]
    # the shapes compiled for three CTAs per multiprocessor (4: 16x16 with
    # the halo warp, 5: 32x8) and the 32x16 tile (6) give the same bits
    batch.set_shape(4, model=0)
    batch.set_shape(5, model=1)
    batch.set_shape(6, model=2)
    assert batch.shape(0) == (16, 16) and batch.shape(1) == (32, 8) and batch.shape(2) == (32, 16)
    for s in solo:
        s.run(4)
    batch.run(4)
    _check_equal(solo, inb)
    batch.close()


def test_batch_production_limiting_matches_individual_runs(built):
    """Characteristic limiting, MULTID shock flattening and ENTROPY_SWITCH
    ALWAYS (the numerics of the production wind configuration) with cooling
    and the line force: the batch's FlagShock pass, PLM and entropy
    recovery give what each model gives alone."""
    import psgb
    kw = dict(cooling=1, line_force=1, char_limiting=1, shock_flattening=1, entropy_switch=2)
    solo = [psgb.wind_model_solver(s, **kw) for s in SPECS]
    inb = [psgb.wind_model_solver(s, **kw) for s in SPECS]
    batch = psgb.Batch(inb)
    # the autotuner's default, then the shapes compiled for two CTAs per
    # multiprocessor (4: 16x16 with the halo warp, 5: 32x8) and the 32x16
    # tile (6), which the characteristic kernels use
    for chunk, shape in ((5, None), (4, 4), (4, 5), (8, 6)):
        if shape is not None:
            batch.set_shape(shape)
        flags = 0
        for s in solo:
            flags |= s.run(chunk)
        assert batch.run(chunk) == flags
        _check_equal(solo, inb)
    batch.close()


def test_batch_ode_cooling_matches_individual_runs(built):
    """The ODE cooling path in a batch (one launch for every model's
    CoolingSource, each model's own dt_cool) gives what each model gives
    alone."""
    import psgb
    solo = [psgb.wind_model_solver(s, cooling=2, line_force=1) for s in SPECS]
    inb = [psgb.wind_model_solver(s, cooling=2, line_force=1) for s in SPECS]
    batch = psgb.Batch(inb)
    for chunk in (5, 8):
        flags = 0
        for s in solo:
            flags |= s.run(chunk)
        assert batch.run(chunk) == flags
        _check_equal(solo, inb)
    batch.close()


def test_batch_state_transfer(built):
    """ps_batch_set_states / ps_batch_get_states move every model's Data.Vc
    in one queue: what they read equals each model's ps_get_state, and a
    batch stepped from states handed in equals the models stepped alone
    from the same states."""
    import psgb
    import torch
    solo, inb = _pairs(1)
    batch = psgb.Batch(inb)
    batch.run(3)
    host = [np.zeros_like(m.get_state()) for m in inb]   # pageable: the copy engines
    batch.get_states(host)
    pinned = [torch.zeros(h.shape, dtype=torch.float64).pin_memory().numpy() for h in host]
    batch.get_states(pinned)                             # pinned: the copy kernel
    for m, h, q in zip(inb, host, pinned):
        assert np.array_equal(h, m.get_state()) and np.array_equal(q, h)
    for s in solo:
        s.run(3)
    # hand in states changed on the host, then step both forms
    for h, q in zip(host, pinned):
        h[4] *= 1.01                 # pressure
        q[...] = h
    batch.set_states(pinned)
    for s, h in zip(solo, host):
        s.set_state(h)
    flags = 0
    for s in solo:
        flags |= s.run(4)
    assert batch.run(4) == flags
    _check_equal(solo, inb)
    batch.close()


def test_batch_overlapped_halves(built):
    """Two batches on their own streams, each step handed in and out through
    pinned host arrays by the queued copy-engine transfers
    (ps_batch_set_states_async / ps_batch_get_states_async) while the other
    batch steps: the same states as the models stepped alone."""
    import psgb
    import torch
    solo, inb = _pairs(1)
    parts = [psgb.Batch(inb[:1]), psgb.Batch(inb[1:])]
    hosts = [[torch.from_numpy(m.get_state()).pin_memory().numpy() for m in p.solvers]
             for p in parts]
    for step in range(6):
        for p, h in zip(parts, hosts):
            p.sync()                   # this part's previous result is on the host
            p.set_states_async(h)
            p.run(1, wait=False)
            p.get_states_async(h)
    flags = 0
    for p in parts:
        flags |= p.sync()
    solo_flags = 0
    for s in solo:
        solo_flags |= s.run(6)
    assert flags == solo_flags
    _check_equal(solo, inb)
    for m, h in zip(inb, hosts[0] + hosts[1]):
        assert np.array_equal(h, m.get_state())
    for p in parts:
        p.close()


def test_batch_rejects_mixed_models(built):
    """Models of one batch share the kernels: cooling kind, limiting form
    and variable count must agree."""
    import psgb
    for kw_a, kw_b in [(dict(cooling=1), dict(cooling=0)),
                       (dict(cooling=1), dict(cooling=2)),
                       (dict(char_limiting=1), dict()),
                       (dict(entropy_switch=2), dict())]:
        a = psgb.wind_model_solver(SPECS[0], **kw_a)
        b = psgb.wind_model_solver(SPECS[1], **kw_b)
        with pytest.raises(RuntimeError):
            psgb.Batch([a, b])
        a.close()
        b.close()
