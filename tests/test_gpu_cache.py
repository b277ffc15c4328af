"""Radiance cache network on the tensor cores against its NumPy restatement
(tests/nrc_reference.py): inference, and the gradients of one training step
(weights and hash table); and that training reduces the loss."""

import numpy as np
import pytest

from path_gb300 import api

import nrc_reference as ref

pytestmark = pytest.mark.gpu

LO, HI = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)


def _queries(rng, n):
    pos = rng.uniform(-1, 1, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    alb = rng.uniform(0, 1, (n, 3))
    return np.concatenate([pos, d, nrm, alb], 1).astype(np.float32)


def _cache(seed=3):
    c = api.RadianceCache(seed=seed)
    c.set_bounds(LO, HI)
    w, t = c.get()
    # larger table features so the encoding matters
    rng = np.random.default_rng(seed)
    t = rng.uniform(-0.5, 0.5, t.shape).astype(np.float32)
    c.set(table=t)
    return c, w, t


@pytest.mark.parametrize("n", [1, 129, 1000])
def test_inference_matches_numpy(lib, n):
    rng = np.random.default_rng(1)
    c, w, t = _cache()
    q = _queries(rng, n)
    got = c.query(q)
    want, _, _, _ = ref.forward(q, w, t, LO, HI)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    print(f"inference rel err {err:.2e}")
    assert err < 1e-2


def test_training_gradients_match_numpy(lib):
    rng = np.random.default_rng(2)
    c, w, t = _cache()
    q = _queries(rng, 700)
    target = rng.uniform(0, 2, (700, 3)).astype(np.float32)
    rec = np.concatenate([q, target, np.zeros((700, 1), np.float32)], 1)
    loss = c.train(rec, update=False)
    _, _, gw, gt = c.get(grads=True)
    loss_ref, gw_ref, gt_ref = ref.gradients(rec, w, t, LO, HI)
    ew = np.linalg.norm(gw - gw_ref) / np.linalg.norm(gw_ref)
    et = np.linalg.norm(gt - gt_ref) / np.linalg.norm(gt_ref)
    print(f"loss {loss:.5f} (numpy {loss_ref:.5f}); weight grad rel err {ew:.2e}, "
          f"table grad rel err {et:.2e}")
    assert abs(loss - loss_ref) / loss_ref < 1e-2
    assert ew < 2e-2
    assert et < 2e-2


def test_training_reduces_the_loss(lib):
    rng = np.random.default_rng(4)
    c = api.RadianceCache(seed=5)
    c.set_bounds(LO, HI)
    q = _queries(rng, 1 << 14)
    # a smooth target radiance field
    p = q[:, :3]
    target = np.stack([1 + np.sin(3 * p[:, 0]), 1 + np.cos(2 * p[:, 1]),
                       1 + 0.5 * p[:, 2] * q[:, 9]], 1).astype(np.float32)
    rec = np.concatenate([q, target, np.zeros((len(q), 1), np.float32)], 1)
    losses = [c.train(rec) for _ in range(200)]
    print(f"loss {losses[0]:.4f} -> {losses[-1]:.4f}")
    assert losses[-1] < 0.1 * losses[0]


def _cornell(w, h, depth=6):
    from path_gb300 import scenes
    sc = scenes.cornell_box()
    s = scenes.path_settings(depth, "wide")
    s.kernel_approach = 1
    return sc, s, scenes.cornell_camera(w, h)


def _render(r, sc, s, f2w, w, h, spp, offset=0):
    out = np.zeros((h, w, 3), np.float32)
    r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w, sample_offset=offset), out, sc,
             spp, s)
    return out


def test_frames_with_sample_offsets_average_to_one_render(lib):
    """Frame f renders Sobol samples [4f, 4f + 4): the mean of frames is the
    render of all their samples (up to the order of the float sums)."""
    sc, s, f2w = _cornell(32, 32)
    r = api.Renderer()
    frames = [_render(r, sc, s, f2w, 32, 32, 4, 4 * f) for f in range(4)]
    whole = _render(r, sc, s, f2w, 32, 32, 16)
    np.testing.assert_allclose(np.mean(frames, 0), whole, rtol=2e-5, atol=1e-6)


def test_trained_cache_lowers_the_error_of_a_frame(lib):
    """What the trained network gains: after training frames, a 4-spp frame
    whose paths end into the cache after 2 bounces is closer to a 1024-spp
    render than a plain 4-spp frame of the same samples."""
    w = h = 64
    sc, s, f2w = _cornell(w, h, depth=8)
    r = api.Renderer()
    ref = _render(r, sc, s, f2w, w, h, 1024)
    cache = api.RadianceCache(seed=7)
    for f in range(40):
        img = np.zeros((h, w, 3), np.float32)
        r.render_cached(cache, api.SquareImage(w, h, f2w, sample_offset=1024 + 4 * f), img, sc,
                        4, s, cache_depth=2, train_paths=1 << 14, train_steps=4)
    spec = api.SquareImage(w, h, f2w, sample_offset=4096)
    cached = np.zeros((h, w, 3), np.float32)
    r.render_cached(cache, spec, cached, sc, 4, s, cache_depth=2, train_paths=0)
    plain = np.zeros((h, w, 3), np.float32)
    r.render(api.ExecutionModel.GPU, spec, plain, sc, 4, s)

    def rel(a):
        return float(np.linalg.norm(a - ref) / np.linalg.norm(ref))

    e_plain, e_cached = rel(plain), rel(cached)
    print(f"4-spp frame rel RMSE: plain {e_plain:.4f}, with trained cache {e_cached:.4f}")
    assert np.isfinite(cached).all()
    assert e_cached < e_plain


def test_moving_average_of_the_parameters_for_inference(lib):
    """With the moving average on, queries read avg = d avg + (1 - d) param
    (starting from the parameters), updated after each Adam step: checked
    against the NumPy network on the average of the parameters before and
    after one step."""
    rng = np.random.default_rng(8)
    c, w0, t0 = _cache(seed=6)
    q = _queries(rng, 600)
    before = c.query(q)
    c.set_ema(0.75)
    assert np.array_equal(c.query(q), before)
    target = rng.uniform(0, 2, (4096, 3)).astype(np.float32)
    rec = np.concatenate([_queries(rng, 4096), target, np.zeros((4096, 1), np.float32)], 1)
    c.train(rec)
    w1, t1 = c.get()
    d = np.float32(0.75)
    wa = d * w0 + (np.float32(1) - d) * w1
    ta = d * t0 + (np.float32(1) - d) * t1
    want, _, _, _ = ref.forward(q, wa, ta, LO, HI)
    got = c.query(q)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    print(f"moving-average inference rel err {err:.2e}")
    assert err < 1e-2
    c.set_ema(0.0)
    live, _, _, _ = ref.forward(q, w1, t1, LO, HI)
    assert np.linalg.norm(c.query(q) - live) / np.linalg.norm(live) < 1e-2
