"""Golden fixtures (tests/golden/*.npz, written by make_golden.py): records
and raw gradient accumulations of small seeded workloads from the FP64
oracle.  The oracle reproduces them (CPU); the FP32 engine matches them
within a relative L2 error of 1e-5 (GPU)."""
import os

import numpy as np
import pytest

from geophyinv_gb300 import L2DistLoss, Recs, get_modelvector, gradient, update

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5


def _cases():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MG = _cases()
NAMES = sorted(MG.cases())


def rel(a, b):
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def _golden(name):
    with np.load(os.path.join(HERE, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_the_golden_fixture(name):
    wl, kind = MG.cases()[name]
    got = MG.compute(wl, kind)
    want = _golden(name)
    assert sorted(got) == sorted(want)
    for k in want:
        assert rel(got[k], want[k]) < 1e-6, (name, k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_engine_matches_the_golden_fixture(engine, name):
    wl, kind = MG.cases()[name]
    want = _golden(name)
    if kind == "forward":
        pa = wl.expt()
        update(pa)
        for f in wl.rfields:
            got = np.stack([pa.data[0][i].d[f] for i in range(len(wl.shots))])
            assert rel(got, want["rec_" + f]) < TOL, (name, f)
        return
    pa = wl.expt(mode="forward_save")
    nr = len(wl.shots[0][1])
    dobs = [Recs(nr, pa.tgrid, list(wl.rfields), {f: np.zeros((wl.nt, nr), np.float32) for f in wl.rfields})
            for _ in wl.shots]
    m = get_modelvector(pa, ["invK", "rho"])
    loss = gradient(np.zeros_like(m), m, L2DistLoss(), dobs, pa)
    assert abs(loss - float(want["loss"][0])) <= 1e-5 * abs(float(want["loss"][0]))
    for k in ("invK", "rho"):
        assert rel(pa.gradients[k], want["grad_" + k]) < TOL, (name, k)
