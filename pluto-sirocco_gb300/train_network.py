"""Train the learned cooling step for a line-driven wind and save the
network for the drop-in (PS_LEARNED_COOLING=<file>, read by ps_sg_load).

    python pluto-sirocco_gb300/train_network.py --grid 512 256 --l-star 1e37 \\
        --krad 0.2 --alpharad -0.6 --out wind.psg

The wind is run on the GPU with the reference cooling step and its cells
are collected at a few step numbers (ps_sg_collect); together with
log-uniform draws over the BLONDIN inputs they are labelled by the
reference method on the GPU and the network is trained there (Adam), as
the benchmark trains its network.  The box of the network is the bounding
box of the training set; cells outside it, and every cell the Newton judge
rejects, are left to the reference method at run time, so a network is
never a correctness risk, only a speed one.  Needs a GPU.
"""
import argparse
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import numpy as np  # noqa: E402

import psgb  # noqa: E402


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--grid", type=int, nargs=2, default=(512, 256), metavar=("NR", "NTHETA"))
    ap.add_argument("--l-star", type=float, default=1e37, help="L_star [erg/s]")
    ap.add_argument("--krad", type=float, default=0.2)
    ap.add_argument("--alpharad", type=float, default=-0.6)
    ap.add_argument("--steps", type=int, nargs="+", default=[0, 40, 120, 240],
                    help="step numbers at which the wind's cells are collected")
    ap.add_argument("--per-snapshot", type=int, default=20000,
                    help="cells drawn from each collected snapshot")
    ap.add_argument("--draws", type=int, default=1000000,
                    help="log-uniform draws over the BLONDIN inputs")
    ap.add_argument("--train-steps", type=int, default=40000)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--out", required=True, help="network file to write")
    a = ap.parse_args(argv)

    spec = dict(grid=tuple(a.grid), l_star=a.l_star, krad=a.krad, alpharad=a.alpharad)
    t0 = time.perf_counter()
    wind = psgb.wind_training_tuples([spec], steps=tuple(a.steps), per_model=a.per_snapshot,
                                     seed=a.seed)
    sg, hist, tup, _ = psgb.train_surrogate(wind, n_draws=a.draws, steps=a.train_steps,
                                            batch=8192, seed=a.seed)
    sg.save(a.out)
    # how the network does on the wind's own cells
    sg.stats(reset=True)
    out, st, _ = sg.predict(wind, use_net=1)
    ref = sg.label(wind)
    ok = ref >= 1e4
    rel = np.abs(out[ok] - ref[ok]) / ref[ok]
    print(f"network written to {a.out}: {len(tup)} training tuples ({len(wind)} from the "
          f"wind), final loss {hist[-100:].mean():.3e}, on the wind's cells "
          f"{np.mean(st == 0):.4f} accepted by the judge, max relative T error "
          f"{rel.max():.2e}; {time.perf_counter() - t0:.1f} s")
    sg.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
