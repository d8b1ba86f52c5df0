"""Source illumination (illum_flag of PFdtd, src/fdtd/fdtd.jl:59,177;
compute_illum!, src/fdtd/fdtd.jl:571-582, at the end of every step,
src/fdtd/propagate.jl:236; stack_illums!, src/fdtd/fdtd.jl:556-566): the
engine's sum over shots and steps of p^2 (square in FP32, sums in FP64) on
the physical grid equals the oracle's (relative L2 < 1e-5) and, bit for
bit, the sum formed from the engine's own snapshots; every run starts from
zero; graph replays give the same sums.  The oracle's sums equal those
formed from its own snapshots (CPU).  The reference declares the flag but
leaves both calls commented out."""
import numpy as np
import pytest

from geophyinv_gb300 import configs, update
from oracle import oracle as O

TOL = 1e-5


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (nb if nb > 0 else 1.0)


def _inner(wl, pa):
    """Slices of the physical grid inside the extended one."""
    out = []
    names = ("z", "y", "x") if wl.ndim == 3 else ("z", "x")
    for ax, nm in enumerate(names):
        lo = pa.npml if nm + "min" in pa_faces(pa) else 0
        n = len(pa.exgrid[ax])
        hi = n - (pa.npml if nm + "max" in pa_faces(pa) else 0)
        out.append(slice(lo, hi))
    return tuple(out)


def pa_faces(pa):
    from geophyinv_gb300 import setup as S

    return [f for f, b in S.FACE_BITS.items() if pa.pml_mask & b]


def _stack(snaps, sl):
    """sum over shots (from 0, shot order) of sum over steps of p^2."""
    tot = None
    for per in snaps:
        acc = np.zeros(per[0][sl].shape, np.float64)
        for p in per:
            q = np.asarray(p[sl], np.float32)
            acc = acc + (q * q).astype(np.float64)
        tot = acc if tot is None else tot + acc
    return tot


def test_oracle_illumination_is_the_sum_of_its_snapshots():
    wl = _two_shots(configs.acoustic2d_layers(nz=30, nx=40, nt=48, nrec=5))
    wl.pml_faces = ["zmax", "xmin", "xmax"]
    res = O.forward(wl.as_dict(), snaps=("p", list(range(1, wl.nt + 1))), illum=True)
    npml = 43  # padded faces: zmax, xmin, xmax
    assert res["illum"].shape == (30, 40)
    assert np.linalg.norm(res["illum"]) > 0
    assert np.array_equal(res["illum"], _stack(res["snaps"], (slice(0, 30), slice(npml, npml + 40))))


def _two_shots(wl):
    src, rec = wl.shots[0]
    xm = wl.grid[-1].last
    wl.shots = [(np.array([[src[0, 0]] + list(src[0, 1:-1]) + [x]]), rec) for x in (0.3 * xm, 0.7 * xm)]
    return wl


@pytest.mark.gpu
@pytest.mark.parametrize("faces", ["all", "free_top"])
def test_acoustic2d_illumination_matches_oracle(engine, faces):
    wl = _two_shots(configs.acoustic2d_layers(nz=60, nx=90, nt=150, nrec=15))
    if faces == "free_top":
        wl.pml_faces = ["zmax", "xmin", "xmax"]
    res = O.forward(wl.as_dict(), illum=True)
    pa = wl.expt(illum_flag=True)
    update(pa)
    got = pa.illum_stack
    assert got.shape == (len(wl.grid[0]), len(wl.grid[1])) and got.dtype == np.float64
    want = res["illum"]
    assert np.linalg.norm(want) > 0
    e = rel(got, want)
    assert e < TOL, e
    assert np.array_equal(pa["illum"], got)


@pytest.mark.gpu
def test_acoustic3d_illumination_matches_oracle(engine):
    wl = configs.acoustic3d(nz=20, ny=18, nx=22, nt=80, npml=10, nrec_side=3, rfields=("p",))
    res = O.forward(wl.as_dict(), illum=True)
    pa = wl.expt(illum_flag=True)
    update(pa)
    e = rel(pa.illum_stack, res["illum"])
    assert e < TOL, e


@pytest.mark.gpu
@pytest.mark.parametrize("order", [4, 2])
def test_illumination_equals_the_sum_of_the_engines_own_snapshots(engine, order):
    wl = _two_shots(configs.acoustic2d_layers(nz=50, nx=70, nt=90, nrec=11))
    tg = wl.tgrid.values()
    pa = wl.expt(illum_flag=True, tsnaps=list(tg), snaps_field="p", order=order)
    assert pa.itsnaps == list(range(1, wl.nt + 1))
    update(pa)
    got = pa.illum_stack
    snaps = [pa["snaps", iss] for iss in range(len(wl.shots))]
    assert np.array_equal(got, _stack(snaps, _inner(wl, pa)))
    # initialize!: every run starts from zero
    update(pa)
    assert np.array_equal(pa.illum_stack, got)


@pytest.mark.gpu
@pytest.mark.parametrize("gkind", [1, 2])
def test_illumination_under_graph_replays(engine, gkind):
    wl = _two_shots(configs.acoustic2d_layers(nz=64, nx=80, nt=100, nrec=11))
    plain = wl.expt(illum_flag=True)
    update(plain)
    pa = wl.expt(illum_flag=True)
    pa.set_graph(gkind)
    for _ in range(2):
        update(pa)
        assert np.array_equal(pa.illum_stack, plain.illum_stack)


@pytest.mark.gpu
def test_illumination_keywords(engine):
    wl = configs.elastic2d_batch(nz=40, nx=60, nt=20, nshots=1, nrec=5)
    with pytest.raises(ValueError):
        wl.expt(illum_flag=True)
    pa = wl.expt(jobname="survey", backprop_flag="save", nworker=1)
    assert pa.jobname == "survey" and not pa.illum_flag
    with pytest.raises(ValueError):
        pa.illum_stack
