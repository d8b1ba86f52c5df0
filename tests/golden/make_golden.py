"""Writes the golden fixtures of tests/test_golden.py: records (and raw
gradient accumulations) of small seeded workloads computed by the CPU
oracle in FP64 (the C restatement of the reference time loop).  The
reference itself (Julia) cannot run here and ships no golden vectors, so
these fix the oracle's answer for regression and let the GPU tests check
the engine against stored FP64 values.

    python tests/golden/make_golden.py      # rewrites tests/golden/*.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "geophyinv.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from geophyinv_gb300 import configs  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cases():
    """name -> (workload, kind): the same builders the tests use."""
    return {
        "acoustic2d_101x131_500": (configs.acoustic2d_layers(nz=101, nx=131, nt=500, nrec=41), "forward"),
        "elastic2d_110x190_2shots_400": (configs.elastic2d_batch(nz=110, nx=190, nt=400, nshots=2, nrec=31),
                                         "forward"),
        "acoustic3d_20x18x22_100": (configs.acoustic3d(nz=20, ny=18, nx=22, nt=100, npml=10, nrec_side=4,
                                                       rfields=("p", "vz")), "forward"),
        "gradient2d_40x70_300": (configs.acoustic2d_fwi(nz=40, nx=70, nt=300, nshots=1, nrec=23, anomaly=False),
                                 "gradient"),
    }


def compute(wl, kind):
    ex = wl.as_dict()
    if kind == "forward":
        res = O.forward(ex, dtype=np.float64)
        return {"rec_" + f: res[f].astype(np.float32) for f in wl.rfields}
    nr = len(wl.shots[0][1])
    dobs = {f: np.zeros((len(wl.shots), wl.nt, nr), np.float64) for f in wl.rfields}
    loss, _, dcal, raw = O.gradient(ex, dobs, dtype=np.float64)
    out = {"rec_" + f: dcal[f].astype(np.float32) for f in wl.rfields}
    out.update({"grad_" + k: v.astype(np.float32) for k, v in raw.items()})
    out["loss"] = np.array([loss])
    return out


if __name__ == "__main__":
    for name, (wl, kind) in cases().items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **compute(wl, kind))
        print("wrote", name)
