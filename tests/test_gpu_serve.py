"""Serving loop: jobs admitted by slots and an HBM budget, their candidates
scored together in shared engine launches, return exactly the poses they
return when run alone; admission keeps the reserved bytes under the budget."""
import numpy as np
import pytest

from autoscoper_gb300 import api, serve

pytestmark = pytest.mark.gpu

RENDER = (192, 192)


def _jobs():
    rng = np.random.default_rng(3)
    subjects = ["a", "b", "a", "c"]
    out = []
    for i, s in enumerate(subjects):
        out.append(serve.make_job(i, rng, s, arrival=0.0, vol_range=(48, 80), view_range=(128, 192), bones=(1, 2),
                                  views=(1, 3), frames=(1, 3), particles=(32, 48), iterations=6,
                                  render_targets=api.render_targets))
    return out


def test_results_same_alone_and_in_mix():
    alone = _jobs()
    launches_alone = 0
    for j in alone:
        srv = serve.Server(hbm_budget=150e9, max_jobs=1, render=RENDER, max_items=512)
        launches_alone += srv.serve([j], realtime=False)["launches"]
    mixed = _jobs()
    srv = serve.Server(hbm_budget=150e9, max_jobs=4, render=RENDER, max_items=512)
    summary = srv.serve(mixed, realtime=False)
    assert summary["failed"] == 0, [j.error for j in mixed]
    assert summary["cache_hits"] >= 1  # subject "a" twice
    # the jobs shared launches: far fewer than the jobs alone needed
    assert summary["launches"] < 0.6 * launches_alone, (summary["launches"], launches_alone)
    for a, m in zip(alone, mixed):
        assert a.error is None and m.error is None
        assert len(a.poses) == len(m.poses) == a.frames
        for pa, pm in zip(a.poses, m.poses):
            assert np.array_equal(pa, pm)
        assert a.evals == m.evals


def test_registration_moves_towards_truth():
    job = _jobs()[1]
    serve.Server(hbm_budget=150e9, max_jobs=1, render=RENDER, max_items=512).serve([job], realtime=False)
    truth = np.array([np.asarray(t, np.float64) for t in job.scene.truth])
    start = np.array([np.asarray(p, np.float64) for p in job.scene.poses])
    final = job.poses[-1]
    assert np.abs(final[:, :3] - truth[:, :3]).mean() < np.abs(start[:, :3] - truth[:, :3]).mean()


def test_admission_respects_budget():
    jobs = _jobs()
    probe = serve.Server(hbm_budget=150e9, max_jobs=4, render=RENDER, max_items=512)
    need = max(sum(serve.volume_bytes(v) for v in j.scene.volumes) + serve.job_bytes(j) for j in jobs)
    budget = probe.base_bytes + 1.5 * need  # room for about one job at a time
    del probe
    srv = serve.Server(hbm_budget=budget, max_jobs=4, render=RENDER, max_items=512)
    summary = srv.serve(jobs, realtime=False)
    assert summary["failed"] == 0, [j.error for j in jobs]
    assert srv.peak <= budget


def test_saturation_cap_admits_no_job_beside_a_full_batch():
    """sat_items: a job joins running ones only while their candidates per
    PSO iteration stay below the cap; with a cap below any job's own, jobs run
    one at a time (as FIFO, in as many launches), with the same poses."""
    fifo = _jobs()
    n_fifo = serve.Server(hbm_budget=150e9, max_jobs=1, render=RENDER, max_items=512).serve(fifo, realtime=False)
    capped = _jobs()
    srv = serve.Server(hbm_budget=150e9, max_jobs=4, render=RENDER, max_items=512, sat_items=1)
    n_cap = srv.serve(capped, realtime=False)
    assert n_cap["failed"] == 0 and n_cap["launches"] == n_fifo["launches"], (n_cap, n_fifo)
    for a, b in zip(fifo, capped):
        for pa, pb in zip(a.poses, b.poses):
            assert np.array_equal(pa, pb)


def test_backlog_rule_runs_jobs_one_at_a_time_without_a_queue():
    """min_backlog: with more waiting jobs required than the stream ever
    holds, the merged loop runs the jobs one at a time (as FIFO), with the
    same poses."""
    fifo = _jobs()
    n_fifo = serve.Server(hbm_budget=150e9, max_jobs=1, render=RENDER, max_items=512).serve(fifo, realtime=False)
    held = _jobs()
    n_held = serve.Server(hbm_budget=150e9, max_jobs=4, render=RENDER, max_items=512,
                          min_backlog=len(held) + 1).serve(held, realtime=False)
    assert n_held["failed"] == 0 and n_held["launches"] == n_fifo["launches"], (n_held, n_fifo)
    for a, b in zip(fifo, held):
        for pa, pb in zip(a.poses, b.poses):
            assert np.array_equal(pa, pb)
