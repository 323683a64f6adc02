"""GPU parity of the batched engine and of the plain per-pose path against
the FP64 oracle's Tracker::minimizationFunc, at the NCC bar: each view's NCC
within 1e-5 relative, 1e-7 absolute where |NCC| < 0.01 (FP32 image rounding
leaves ~1e-8 of NCC per stage); a cost, the sum over views of 1 - NCC,
within the sum of its views' bars.  SAD costs within 1e-5 relative."""
import numpy as np
import pytest

from autoscoper_gb300 import _lib as L
from autoscoper_gb300 import api, scene as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_REL = 1e-5
NCC_FLOOR = 1e-2  # below |NCC| = 0.01 the bar is the absolute TOL_REL * NCC_FLOOR
TOL_ABS_SAD = 2e-6  # SAD costs: FP32 tile partials of |(f - mF) - (g - mG)|


def ncc_bar(ncc):
    return TOL_REL * max(abs(ncc), NCC_FLOOR)


def make_targets(sc, tr):
    for vi, v in enumerate(sc.views):
        drr_sum = np.zeros((v.camera.height, v.camera.width))
        for b in range(len(sc.volumes)):
            ok, m, _, _, _ = tr.view_setup(b, vi, sc.truth[b])
            rp = sc.ray[vi][b]
            drr_sum += O.raycast(tr.vd[b], m, S.target_viewport(v.camera), rp.step, rp.intensity, rp.cutoff,
                                 v.camera.width, v.camera.height)
        v.radiograph = S.radiograph_from_drr(drr_sum, seed=vi)


@pytest.fixture(scope="module", params=["sobel", "chain"])
def scene(request):
    sc = S.make_scene([(40, 48, 56), (36, 30, 44)], 1.0, (112, 112), 0.9, filters=request.param, seed=7,
                      bone_offsets=[(0, 0, -12), (4, -3, 14)])
    tr = O.Tracker(sc)
    make_targets(sc, tr)
    return sc, tr


def _cands(rng, n, nb, spread=2.0):
    bones = rng.integers(0, nb, n).astype(np.int32)
    man = np.concatenate([rng.uniform(-spread, spread, (n, 3)), rng.uniform(-spread, spread, (n, 3))], 1)
    man[0] = 0
    return bones, man


def _check(got, ref, refv):
    """A cost against the oracle's: within the sum of its views' NCC bars
    (refv: the oracle's per-view terms 1 - NCC; a 9999 term is exact)."""
    bar = sum(ncc_bar(1.0 - c) if c != 9999.0 else 0.0 for c in refv)
    assert abs(got - ref) <= bar, (got, ref, bar)


@pytest.mark.parametrize("coverage", [L.ASC_SUM_TREE, L.ASC_SUM_FULL])
def test_engine_and_plain_match_oracle(scene, coverage):
    sc, tr0 = scene
    tr = O.Tracker(sc, tree=coverage == L.ASC_SUM_TREE)
    eng = api.Engine(sc, max_items=32, coverage=coverage)
    rng = np.random.default_rng(11)
    bones, man = _cands(rng, 12, len(sc.volumes))
    cost, vcost = eng.eval(bones, man)
    pcost, pvcost = eng.eval(bones, man, plain=True)
    for k in range(len(bones)):
        ref = tr.minimization_func(int(bones[k]), man[k])
        refv = tr.track_frame(int(bones[k]), tr.compose(int(bones[k]), man[k]))
        # cost = sum over views of (1 - NCC): each term within the NCC bar
        _check(cost[k], ref, refv)
        _check(pcost[k], ref, refv)
        for v in range(2):
            for got in (vcost[k, v], pvcost[k, v]):
                n_got, n_ref = 1.0 - got, 1.0 - refv[v]
                assert abs(n_got - n_ref) <= ncc_bar(n_ref), (n_got, n_ref)


@pytest.mark.parametrize("coverage", [L.ASC_SUM_TREE, L.ASC_SUM_FULL])
def test_engine_sad_cost_model_matches_oracle(scene, coverage):
    """cf_model 1 (Tracker.cpp:762-766): each view scores the SAD of
    gpu::hdist, batched (k_view then k_sad) and plain, against the oracle;
    per view within 1e-5 relative of the SAD."""
    import copy
    sc = copy.copy(scene[0])
    sc.cf_model = 1
    tr = O.Tracker(sc, tree=coverage == L.ASC_SUM_TREE)
    eng = api.Engine(sc, max_items=32, coverage=coverage)
    rng = np.random.default_rng(21)
    bones, man = _cands(rng, 12, len(sc.volumes))
    man[-1] = [0, 0, 5000.0, 0, 0, 0]  # out of view: 9999 per view
    cost, vcost = eng.eval(bones, man)
    pcost, pvcost = eng.eval(bones, man, plain=True)
    for k in range(len(bones)):
        refv = tr.track_frame(int(bones[k]), tr.compose(int(bones[k]), man[k]))
        ref = tr.minimization_func(int(bones[k]), man[k])
        assert ref == pytest.approx(sum(refv))
        for got in (cost[k], pcost[k]):
            assert abs(got - ref) <= TOL_REL * abs(ref) + TOL_ABS_SAD, (got, ref)
        for v in range(2):
            assert refv[v] > 0
            for got in (vcost[k, v], pvcost[k, v]):
                assert abs(got - refv[v]) <= TOL_REL * refv[v] + TOL_ABS_SAD, (k, v, got, refv[v])
    assert np.all(vcost[-1] == 9999.0)
    # the batch is order independent in this mode too
    perm = rng.permutation(len(bones))
    c2, _ = eng.eval(bones[perm], man[perm])
    assert np.array_equal(cost[perm], c2)


def test_engine_out_of_view_penalty(scene):
    sc, tr = scene
    eng = api.Engine(sc, max_items=4)
    man = np.array([[0, 0, 0, 0, 0, 0], [900.0, 0, 0, 0, 0, 0], [0, 0, 5000.0, 0, 0, 0]])
    cost, vcost = eng.eval(np.zeros(3, np.int32), man)
    for k in range(3):
        _check(cost[k], tr.minimization_func(0, man[k]), tr.track_frame(0, tr.compose(0, man[k])))
    assert cost[2] == 2 * 9999.0 and np.all(vcost[2] == 9999.0)  # Tracker.cpp:614-617


def test_engine_batch_is_order_independent(scene):
    sc, tr = scene
    eng = api.Engine(sc, max_items=64)
    rng = np.random.default_rng(12)
    bones, man = _cands(rng, 40, len(sc.volumes))
    c1, _ = eng.eval(bones, man)
    perm = rng.permutation(len(bones))
    c2, _ = eng.eval(bones[perm], man[perm])
    single = np.array([eng.eval(bones[k:k + 1], man[k:k + 1])[0][0] for k in range(5)])
    assert np.array_equal(c1[perm], c2)
    assert np.array_equal(c1[:5], single)


def test_engine_empty_space_skipping_changes_no_bit(scene):
    """The occupied-box screen, the DDA walk and the block trimming skip only
    samples that add exactly nothing: costs and DRRs with skipping on equal
    those of the full march, bit for bit."""
    sc, tr = scene
    rng = np.random.default_rng(5)
    bones, man = _cands(rng, 24, len(sc.volumes), spread=4.0)
    try:
        L.call("asc_set_option", L.ASC_OPT_EMPTY_SKIP, 0)
        eng_full = api.Engine(sc, max_items=32)
        full, vfull = eng_full.eval(bones, man)
    finally:
        L.call("asc_set_option", L.ASC_OPT_EMPTY_SKIP, 1)
    eng = api.Engine(sc, max_items=32)
    skip, vskip = eng.eval(bones, man)
    assert np.array_equal(full, skip)
    assert np.array_equal(vfull, vskip)


def test_engine_golden_reference_values():
    """NCC of the reference's own outputs (tests/golden) vs the engine."""
    import golden_scene
    sc, z = golden_scene.load()
    eng = api.Engine(sc, max_items=4)
    poses = z["poses"]
    tr = O.Tracker(sc)
    for k, pose in enumerate(poses):
        sc.poses[0] = np.asarray(pose, np.float32)
        eng.set_base_pose(0, pose)
        tr.scene = sc
        cost, vcost = eng.eval(np.zeros(1, np.int32), np.zeros((1, 6)))
        for vi in range(2):
            ref_ncc = float(z[f"v{vi}p{k}_ncc"])  # reference kernels, float
            # the NCC bar: 1e-5 relative, 1e-7 absolute below |NCC| = 0.01
            assert abs((1.0 - vcost[0, vi]) - ref_ncc) <= 1e-5 * max(abs(ref_ncc), 1e-2), (vi, k, ref_ncc)


def test_pso_converges():
    sc = S.make_scene([(40, 48, 56), (36, 30, 44)], 1.0, (112, 112), 0.9, filters="sobel", seed=9,
                      bone_offsets=[(0, 0, -12), (4, -3, 14)])
    tr = O.Tracker(sc)
    make_targets(sc, tr)
    rng = np.random.default_rng(4)
    sc.poses = [S.perturb(t, rng, 1.5, 1.5) for t in sc.truth]
    eng = api.Engine(sc, max_items=2 * 48)
    best, cost, evals = eng.pso(n_particles=48, n_iter=25, lo=-3, hi=3, seed=3)
    assert evals == 2 * 48 * 25
    for b in range(2):
        c0 = tr.minimization_func(b, np.zeros(6))
        assert cost[b] < c0
        _check(cost[b], tr.minimization_func(b, best[b]), tr.track_frame(b, tr.compose(b, best[b])))
    # the stall rule stops each swarm once its gBest stops moving
    best2, cost2, ev2 = eng.pso(n_particles=48, n_iter=400, lo=-3, hi=3, seed=3, max_stall=3)
    its = eng.last_pso_iterations
    assert 3 <= its < 400
    assert 48 * its <= ev2 <= 2 * 48 * its
    for b in range(2):
        assert cost2[b] < tr.minimization_func(b, np.zeros(6))
        _check(cost2[b], tr.minimization_func(b, best2[b]), tr.track_frame(b, tr.compose(b, best2[b])))


def test_hidden_bone_scores_the_empty_mask(scene):
    """RayCaster::setVisible(false) renders zeros (RayCaster.cpp:131-134): a
    hidden bone's views score the empty-mask cost (1 - 1e5 for NCC) batched
    and plain, its images export a zero DRR and mask, and showing it again
    restores the costs."""
    sc, tr = scene
    eng = api.Engine(sc, max_items=8)
    bones = np.array([0, 1], np.int32)
    man = np.zeros((2, 6))
    before, _ = eng.eval(bones, man)
    eng.set_visible(0, False)
    cost, vcost = eng.eval(bones, man)
    pcost, pvcost = eng.eval(bones, man, plain=True)
    assert np.all(vcost[0] == 1.0 - 1e5) and np.all(pvcost[0] == 1.0 - 1e5)
    assert cost[0] == 9999.0 and pcost[0] == 9999.0  # a negative total is the reference's 9999
    assert cost[1] == before[1]
    rad, drr, mask = eng.image_data(0, 0, np.asarray(sc.poses[0], np.float64))
    assert not drr.any() and not mask.any()
    eng.set_visible(0, True)
    again, _ = eng.eval(bones, man)
    assert np.array_equal(again, before)


def test_launch_shapes_change_no_result(scene):
    """The autotuner's launch shapes (ray-cast blocks per SM, a warp's ray
    block, filter blocks per SM) change times only: every shape gives the
    same costs to the bit."""
    import ctypes as C
    sc, tr = scene
    eng = api.Engine(sc, max_items=32)
    rng = np.random.default_rng(17)
    bones, man = _cands(rng, 24, len(sc.volumes))
    want, wantv = eng.eval(bones, man)
    for cfg in ((4, 0, 2), (3, 1, 4), (2, 2, 3), (1, 1, 2)):
        c = L.LaunchConfig(*cfg)
        L.call("asc_engine_set_launch", eng.handle, C.byref(c))
        got, gotv = eng.eval(bones, man)
        assert np.array_equal(got, want) and np.array_equal(gotv, wantv), cfg
    bad = L.LaunchConfig(5, 0, 3)
    assert L.load().asc_engine_set_launch(eng.handle, C.byref(bad)) == -1


def test_engines_with_different_chains_coexist():
    """k_view's shared-memory limit belongs to the function, not the engine:
    an engine created after one with a wider filter chain must not lower it
    below what the first launches with."""
    wide = S.make_scene([(40, 48, 56)], 1.0, (112, 112), 0.9, filters="chain", seed=3)
    narrow = S.make_scene([(40, 48, 56)], 1.0, (112, 112), 0.9, filters="sobel", seed=3)
    for sc in (wide, narrow):
        make_targets(sc, O.Tracker(sc))
    e_wide = api.Engine(wide, max_items=8)
    man = np.zeros((2, 6))
    man[1] = [0.3, -0.2, 0.1, 0.5, 0.2, -0.4]
    want, _ = e_wide.eval(np.zeros(2, np.int32), man)
    e_narrow = api.Engine(narrow, max_items=8)
    e_narrow.eval(np.zeros(2, np.int32), man)
    got, _ = e_wide.eval(np.zeros(2, np.int32), man)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("coverage", [L.ASC_SUM_TREE, L.ASC_SUM_FULL])
def test_engine_background_threshold_matches_oracle(coverage):
    """View::renderBackground with a threshold >= 0 (View.cpp:171-194,
    BackgroundRenderer_kernels.cu:88-120): the background mask multiplies the
    DRR mask (Tracker.cpp:744-752).  The fused k_view branch and the plain
    path against the oracle, per view within the NCC bar; the mask must cut
    pixels the DRR mask keeps."""
    sc = S.make_scene([(40, 48, 56), (36, 30, 44)], 1.0, (112, 112), 0.9, filters="chain", seed=19,
                      bone_offsets=[(0, 0, -12), (4, -3, 14)])
    tr = O.Tracker(sc)
    make_targets(sc, tr)
    yy, xx = np.mgrid[0:112, 0:112]
    for i, v in enumerate(sc.views):
        v.background = (0.5 + 0.5 * np.sin(xx / (7.0 + i)) * np.cos(yy / 11.0)).astype(np.float32)
        v.bg_threshold = 0.35
    tr = O.Tracker(sc, tree=coverage == L.ASC_SUM_TREE)
    eng = api.Engine(sc, max_items=32, coverage=coverage)
    rng = np.random.default_rng(23)
    bones, man = _cands(rng, 10, len(sc.volumes))
    cost, vcost = eng.eval(bones, man)
    pcost, pvcost = eng.eval(bones, man, plain=True)
    refs = []
    for k in range(len(bones)):
        pose = tr.compose(int(bones[k]), man[k])
        refv = tr.track_frame(int(bones[k]), pose)
        refs.append(refv)
        _check(cost[k], tr.minimization_func(int(bones[k]), man[k]), refv)
        _check(pcost[k], tr.minimization_func(int(bones[k]), man[k]), refv)
        for v in range(2):
            for got in (vcost[k, v], pvcost[k, v]):
                assert abs((1.0 - got) - (1.0 - refv[v])) <= ncc_bar(1.0 - refv[v]), (k, v, got, refv[v])
    # the threshold matters: without it the oracle scores differently
    for v in sc.views:
        v.bg_threshold = -1.0
    plain = [tr.track_frame(int(bones[k]), tr.compose(int(bones[k]), man[k])) for k in range(len(bones))]
    assert not np.allclose(np.array(plain), np.array(refs), rtol=1e-3, atol=0)
