"""Serving loop: jobs admitted by an HBM budget, run concurrently on their
own streams, return exactly the poses they return when run alone."""
import numpy as np
import pytest

from autoscoper_gb300 import api, serve

pytestmark = pytest.mark.gpu


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
    for j in alone:
        serve.Server(hbm_budget=150e9, slots=1).serve([j], realtime=False)
    mixed = _jobs()
    summary = serve.Server(hbm_budget=150e9, slots=4).serve(mixed, realtime=False)
    assert summary["failed"] == 0, [j.error for j in mixed]
    assert summary["cache_hits"] >= 1  # subject "a" twice
    for a, m in zip(alone, mixed):
        assert a.error is None and m.error is None
        assert len(a.poses) == len(m.poses) == a.frames
        for pa, pm in zip(a.poses, m.poses):
            assert np.array_equal(pa, pm)


def test_admission_respects_budget():
    jobs = _jobs()
    need = max(serve.engine_bytes(j.scene, len(j.scene.volumes) * j.particles) for j in jobs)
    budget = 1.5 * need + 2e9  # room for about one job at a time
    srv = serve.Server(hbm_budget=budget, slots=4)
    summary = srv.serve(jobs, realtime=False)
    assert summary["failed"] == 0, [j.error for j in jobs]
    assert srv.peak <= budget
