"""Batched / served engine (emfa_serve).

CPU: the admitter's policy on a simulated clock (emfa_serve_simulate runs
the same choice function as the lanes).
GPU: every request solved in a batch or in a realtime mix gives the same
RCS as the same request solved alone (tolerance 1e-6 dB: the lanes run the
same kernels on their own streams, so the results agree to rounding).
"""
import numpy as np
import pytest

from emfa_gb300 import mesh as M

GB = 1 << 30


def test_admitter_fifo_when_everything_fits(emfa_lib):
    from emfa_gb300 import api
    arr = [0.0, 0.1, 0.2, 0.3]
    start, lane = api.serve_simulate(arr, [1, 1, 1, 1], [GB] * 4, lanes=2, hbm_budget=100 * GB)
    assert np.allclose(start, [0.0, 0.1, 1.0, 1.1])
    assert lane[0] != lane[1]


def test_admitter_budget_lets_small_requests_pass_a_large_one(emfa_lib):
    from emfa_gb300 import api
    # all arrive together: the largest (request 1, 8 GB) starts first; request
    # 0 needs 4 GB with 2 GB free, so the 1 GB requests go ahead of it
    start, _ = api.serve_simulate([0.0, 0.0, 0.0, 0.0], [5, 5, 1, 1], [4 * GB, 8 * GB, GB, GB], lanes=3,
                                  hbm_budget=10 * GB, realtime=False)
    assert start[1] == 0.0 and start[2] == 0.0 and start[3] == 0.0
    assert start[0] == 5.0  # admitted once request 1 gave its 8 GB back


def test_admitter_takes_a_batch_largest_first(emfa_lib):
    from emfa_gb300 import api
    # one lane, everything present at once: by size, largest first; with
    # arrivals apart, by arrival
    start, _ = api.serve_simulate([0.0, 0.0, 0.0], [1, 2, 3], [GB, 3 * GB, 2 * GB], lanes=1, realtime=False)
    assert np.allclose(start, [5.0, 0.0, 2.0])
    start, _ = api.serve_simulate([0.0, 0.1, 0.2], [1, 2, 3], [GB, 3 * GB, 2 * GB], lanes=1, realtime=True)
    assert np.allclose(start, [0.0, 1.0, 3.0])


def test_admitter_oversized_request_runs_alone(emfa_lib):
    from emfa_gb300 import api
    start, _ = api.serve_simulate([0.0, 0.0, 0.5], [2, 1, 1], [20 * GB, GB, GB], lanes=4, hbm_budget=10 * GB)
    # the 20 GB request never fits: it waits until nothing runs, then runs alone
    assert start[1] == 0.0 and start[2] == 0.5
    assert start[0] == pytest.approx(1.5)


def test_admitter_age_limit_keeps_a_large_request_from_starving(emfa_lib):
    from emfa_gb300 import api
    # a 3 GB request every 0.5 s, each running 1 s: two run at any time (6 GB
    # of a 10 GB budget), so the 8 GB request that arrived at 0.2 s never fits
    # while the stream lasts ...
    small = [0.5 * i for i in range(11)]
    arr = [0.2] + small
    dur = [1.0] * len(arr)
    nb = [8 * GB] + [3 * GB] * len(small)
    start, _ = api.serve_simulate(arr, dur, nb, lanes=8, hbm_budget=10 * GB, max_wait_s=1e9)
    assert start[0] > 5.0
    # ... unless, once it has waited max_wait_s, later requests are held back:
    # the small ones of 0.5 s and 1.0 s finish at 1.5 s and 2.0 s, and it starts
    start, _ = api.serve_simulate(arr, dur, nb, lanes=8, hbm_budget=10 * GB, max_wait_s=1.0)
    assert start[0] == pytest.approx(2.0)
    assert all(s >= 3.0 for s, a in zip(start[1:], small) if 1.2 <= a < 3.0)


def test_admitter_honours_arrivals(emfa_lib):
    from emfa_gb300 import api
    arr = [0.0, 2.0, 2.5]
    start, _ = api.serve_simulate(arr, [0.5, 0.5, 0.5], [GB] * 3, lanes=4)
    assert np.allclose(start, arr)
    start, _ = api.serve_simulate(arr, [0.5, 0.5, 0.5], [GB] * 3, lanes=4, realtime=False)
    assert np.allclose(start, 0.0)


def _alone(req_factory, i):
    from emfa_gb300 import api
    r = req_factory()[i]
    r.arrival_s = 0.0
    res = api.serve([r], lanes=1)
    assert res[0].status == 0
    return r.rcs


def test_workloads_sizes():
    from emfa_gb300 import api, workloads as W
    ns = [api.build_rwg(m.tris).shape[0] for (m, f, a, d) in W.batch_set(seed=0, count=64)]
    assert 500 <= min(ns) and max(ns) <= 8000
    st = W.served_stream(seed=0, count=40)
    ns = [api.build_rwg(m.tris).shape[0] for (t, m, f, a, d) in st]
    assert 900 <= min(ns) and max(ns) <= 125000
    ts = [t for (t, m, f, a, d) in st]
    assert all(b > a for a, b in zip(ts, ts[1:]))


@pytest.mark.gpu
def test_batch_each_result_equals_alone(emfa_lib):
    from emfa_gb300 import api, workloads as W
    probs = [W.batch_set(seed=3, count=6, n_inc=3)[i] for i in range(6)]

    def reqs():
        return [api.RcsRequest(m, f, ang, d, kind="efie", per_rhs=True) for (m, f, ang, d) in probs]

    batch = reqs()
    res = api.serve(batch, lanes=3)
    assert all(r.status == 0 for r in res), [r.status for r in res]
    assert all(r.converged == 3 and r.method == 1 for r in res)
    for i in range(len(batch)):
        assert np.abs(batch[i].rcs - _alone(reqs, i)).max() < 1e-6


@pytest.mark.gpu
def test_served_mix_equals_alone_and_timing(emfa_lib):
    """Staggered arrivals of dense and MLFMA requests, overlapping on the
    device: each result matches the request run alone; each request starts
    no earlier than it arrives."""
    from emfa_gb300 import api
    meshes = [(M.icosphere(2, 0.5), 3e8), (M.cube(8, 0.8), 4e8), (M.icosphere(3, 0.5), 3e8),
              (M.icosphere(5, 1.5), 3e8), (M.cube(10, 0.9), 3e8), (M.icosphere(2, 0.4), 5e8)]
    rng = np.random.default_rng(1)
    angs = [np.stack([rng.uniform(0, 180, 2), rng.uniform(0, 360, 2), np.zeros(2)], 1) for _ in meshes]

    def reqs():
        return [api.RcsRequest(m, f, a, api.monostatic_dirs(a), kind="cfie", alpha=0.5, per_rhs=True,
                               arrival_s=0.05 * i)
                for i, ((m, f), a) in enumerate(zip(meshes, angs))]

    mix = reqs()
    res = api.serve(mix, lanes=4, realtime=True, dense_max=10000)
    assert all(r.status == 0 for r in res), [r.status for r in res]
    assert {r.method for r in res} == {1, 2}  # icosphere(5) has 30720 unknowns: MLFMA
    for i, r in enumerate(res):
        assert r.t_start >= r.t_arrive - 1e-9 and r.t_done >= r.t_start
        assert r.converged == 2
    for i in range(len(mix)):
        alone = reqs()[i]
        alone.arrival_s = 0.0
        api.serve([alone], lanes=1, dense_max=10000)
        assert np.abs(mix[i].rcs - alone.rcs).max() < 1e-6, i
