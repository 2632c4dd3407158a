"""Generates the golden fixtures in this directory.

Each fixture is a seeded input (positions, velocities, world, physics) and the
oracle's binned frames after a list of step counts.  The oracle is pinned to
the reference's own known-answer tests (tests/test_oracle_golden.py); these
fixtures freeze its output so that the CUDA path (tests/test_gpu_golden.py)
and the oracle on another machine (tests/test_oracle_props.py) are checked
against the same bits.

Run from the repository root:  python tests/golden/make_fixtures.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

CASES = {
    # reference physics, cell size 3, a dense patch that overflows the
    # capacity of 9 particles per cell
    "reference_48x36_cs3": dict(dims=(48.0, 36.0), cs=3, mode=0, n=1200, vel=0.6, seed=0,
                                patch=200, steps=[1, 10]),
    # extended physics, cell size 1
    "extended_96x64_cs1": dict(dims=(96.0, 64.0), cs=1, mode=1, n=2000, vel=1.0, seed=1,
                               iterations=4, gravity=0.1, steps=[1, 10]),
    # the small configuration's physics at a quarter of its size, 100 steps
    "extended_256_cs1_100": dict(dims=(256.0, 256.0), cs=1, mode=1, n=4096, vel=2.0, seed=0,
                                 iterations=4, gravity=0.1, steps=[100]),
}


def inputs(case):
    rng = np.random.default_rng(case["seed"])
    pos = rng.uniform((0, 0), case["dims"], size=(case["n"], 2)).astype(np.float32)
    vel = rng.normal(0, case["vel"], size=(case["n"], 2)).astype(np.float32)
    if case.get("patch"):
        k = case["patch"]
        pos[:k] = (np.float32(7.5) + rng.uniform(-1, 1, (k, 2))).astype(np.float32)
    return pos, vel


def physics(case):
    if case["mode"] == 0:
        return O.reference_physics()
    return O.extended_physics(case["iterations"], case["gravity"])


def generate(name, case):
    pos, vel = inputs(case)
    w = O.world(case["dims"][0], case["dims"][1], case["cs"])
    table, p, v = O.pack(w, pos, vel, O.max_particles_per_frame(w))
    out = {"pos_in": pos, "vel_in": vel, "table_0": table, "pos_0": p, "vel_0": v}
    done = 0
    for s in case["steps"]:
        table, p, v, _ = O.step(w, physics(case), table, p, v, s - done)
        done = s
        out["table_%d" % s] = table
        out["pos_%d" % s] = p
        out["vel_%d" % s] = v
    meta = dict(case)
    meta["name"] = name
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def load(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    return meta, {k: z[k] for k in z.files if k != "meta"}


if __name__ == "__main__":
    for name, case in CASES.items():
        generate(name, case)
        print("wrote", name)
