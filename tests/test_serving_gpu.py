"""The continuous-batching serving loop: every request's result is the same
alone and in the mix (bit for bit), and the loop keeps several requests on
the device at once."""
import numpy as np
import pytest

from geophyinv_gb300 import serving


def _same(a, b):
    assert a.kind == b.kind
    for ra, rb in zip(a.records, b.records):
        for f in ra:
            assert np.array_equal(ra[f], rb[f]), (a.rid, f)
    if a.gradient is not None:
        for k in a.gradient:
            assert np.array_equal(a.gradient[k], b.gradient[k]), (a.rid, k)
        assert abs(a.loss - b.loss) <= 1e-12 * abs(b.loss)  # summed in another order


@pytest.mark.gpu
def test_results_alone_equal_results_in_the_mix(engine):
    reqs = serving.make_stream(10, rate=1000.0, seed=7, sides=(60, 140), steps=(80, 200), shots=(1, 3))
    assert {r.kind for r in reqs} == set(serving.KINDS)
    mixed, stats = serving.serve(reqs, max_inflight=6, realtime=False)
    assert len(mixed) == len(reqs) and stats["shots"] == sum(r.nshots for r in reqs)
    # overlap: some request was admitted before an earlier one completed
    order = sorted(mixed.values(), key=lambda r: r.t_admit)
    assert any(b.t_admit < a.t_done for a, b in zip(order, order[1:]))
    for r in reqs:
        alone, _ = serving.serve_plain([r], realtime=False)
        _same(mixed[r.rid], alone[r.rid])


@pytest.mark.gpu
def test_admission_respects_the_hbm_budget(engine):
    reqs = serving.make_stream(4, rate=1000.0, seed=3, sides=(60, 100), steps=(50, 80), shots=(1, 2))
    budget = max(serving.request_bytes(r) for r in reqs)  # room for one request at a time
    res, stats = serving.serve(reqs, hbm_budget=budget, max_inflight=4, realtime=False)
    order = sorted(res.values(), key=lambda r: r.t_admit)
    assert all(b.t_admit >= a.t_done for a, b in zip(order, order[1:]))


@pytest.mark.gpu
def test_one_shot_at_a_time_baseline_gives_the_same_results(engine):
    """The baseline's single-shot plans give the same records as the batched
    multi-shot plans of the server (bit for bit), and the same summed
    gradient up to the order of the shot sum."""
    reqs = serving.make_stream(6, rate=1000.0, seed=11, sides=(60, 120), steps=(60, 150), shots=(2, 3))
    mixed, _ = serving.serve(reqs, max_inflight=4, realtime=False)
    single, _ = serving.serve_plain(reqs, realtime=False, per_shot=True)
    for r in reqs:
        a, b = mixed[r.rid], single[r.rid]
        assert len(a.records) == len(b.records) == r.nshots
        for ra, rb in zip(a.records, b.records):
            for f in ra:
                assert np.array_equal(ra[f], rb[f]), (r.rid, f)
        if a.gradient is not None:
            for k in a.gradient:
                ga, gb = a.gradient[k].astype(np.float64), b.gradient[k].astype(np.float64)
                assert np.linalg.norm(ga - gb) <= 1e-6 * np.linalg.norm(gb), (r.rid, k)
            assert abs(a.loss - b.loss) <= 1e-6 * abs(b.loss)
