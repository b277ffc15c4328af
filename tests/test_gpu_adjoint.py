"""Adjoint of the render (path_render_adjoint, path replay): gradients of an
L2 image loss with respect to per-material reflectance, GGX roughness and
emission, checked against central finite differences with common random
numbers (the same Sobol samples: the renders are deterministic), on the
GPU and through the CPU oracle, and through torch.autograd.

Workload: the Cornell geometry split into 16 material patches (Diffuse and
GGX), 128 x 128, 64 spp, depth 4; target rendered from parameters perturbed
by up to 10% (seed 2).

Tolerance: relative error ||g_adjoint - g_fd|| / ||g_fd|| <= 1e-2.
Reflectance and emission do not move any path (the image is smooth in
them), so central differences of step 1e-3 measure the derivative the
adjoint computes.  Roughness moves the directions the GGX sampler draws, so
finite differences then cross visibility and triangle boundaries and are
dominated by O(1/h) jumps; the adjoint differentiates the BSDF with the
sampling held fixed.  Roughness is therefore checked exactly with the
Uniform direction sampler (directions independent of roughness, the image
smooth in it) and, with the BSDF sampler, statistically: step 0.02 at 1024
spp, 0.15 relative.
"""

import time

import numpy as np
import pytest

from path_gb300 import api, capi, diff, scenes

pytestmark = pytest.mark.gpu

W = H = 128
SPP = 64
DEPTH = 4
STEP = 1e-3


def _setup(dir_sampler=0, spp=SPP, rng=0):
    sc, mats = scenes.patch_cornell(seed=1)
    s = scenes.path_settings(DEPTH, "wide")
    s.kernel_approach = 1
    s.dir_sampler = dir_sampler
    s.rng = rng
    spec = api.SquareImage(W, H, scenes.cornell_camera(W, H))
    rend = diff.Renderable(sc, mats, spec, spp, s)
    p0 = diff.params_of(mats)
    target = rend.render(scenes.perturbed_params(p0, mats, seed=2))
    return rend, mats, p0, target


def _loss(img, target):
    d = img.astype(np.float64) - target
    return float((d * d).sum())


def _active(mats):
    """(material, param) pairs with a defined derivative."""
    out = []
    for i, m in enumerate(mats):
        if m.type in (capi.BSDF["Diffuse"], capi.BSDF["GGX"]):
            out += [(i, 0), (i, 1), (i, 2)]
        if m.type == capi.BSDF["GGX"]:
            out.append((i, 3))
        if max(m.emission) > 0:
            out += [(i, 4), (i, 5), (i, 6)]
    return out


def _fd(render, p0, target, pairs, step=STEP):
    g = np.zeros(len(pairs))
    for k, (i, j) in enumerate(pairs):
        pp, pm = p0.copy(), p0.copy()
        pp[i, j] += step
        pm[i, j] -= step
        g[k] = (_loss(render(pp), target) - _loss(render(pm), target)) / (2 * step)
    return g


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("sampler", ["bsdf", "uniform", "bsdf_uniform_rng"])
def test_adjoint_matches_central_differences_on_the_gpu(lib, sampler):
    """bsdf_uniform_rng: the replay re-seeds each path's XORWOW generator, so
    the Uniform RNG gives common random numbers too."""
    rend, mats, p0, target = _setup(dir_sampler=1 if sampler == "uniform" else 0,
                                    rng=1 if sampler == "bsdf_uniform_rng" else 0)
    img = rend.render(p0)
    g_adj = rend.adjoint(p0, (2.0 * (img.astype(np.float64) - target)).astype(np.float32))
    pairs = _active(mats)
    if sampler != "uniform":
        pairs = [pq for pq in pairs if pq[1] != 3]
    g_fd = _fd(rend.render, p0, target, pairs)
    a = np.array([g_adj[i, j] for i, j in pairs])
    err = _rel(a, g_fd)
    print(f"adjoint vs FD ({sampler} sampler): rel err {err:.3e} over {len(pairs)} parameters")
    for (i, j), x, y in zip(pairs, a, g_fd):
        print(f"  mat {i:2d} {diff.PARAMS[j]:9s} adjoint {x: .6e} fd {y: .6e}")
    assert err <= 1e-2


def test_roughness_gradient_with_the_ggx_sampler_statistically(lib):
    rend, mats, p0, target = _setup(spp=1024)
    img = rend.render(p0)
    g_adj = rend.adjoint(p0, (2.0 * (img.astype(np.float64) - target)).astype(np.float32))
    pairs = [(i, 3) for i, m in enumerate(mats) if m.type == capi.BSDF["GGX"]]
    g_fd = _fd(rend.render, p0, target, pairs, step=0.02)
    a = np.array([g_adj[i, j] for i, j in pairs])
    err = _rel(a, g_fd)
    print(f"roughness, GGX sampler, 1024 spp, step 0.02: rel err {err:.3e}")
    for (i, j), x, y in zip(pairs, a, g_fd):
        print(f"  mat {i:2d} roughness adjoint {x: .6e} fd {y: .6e}")
    assert err <= 0.15


def test_adjoint_matches_differences_of_the_oracle(lib, oracle):
    from oracle import oracle_lib as ol
    rend, mats, p0, target = _setup()
    img = rend.render(p0)
    g_adj = rend.adjoint(p0, (2.0 * (img.astype(np.float64) - target)).astype(np.float32))
    st = ol.settings_from(scenes.path_settings(DEPTH, "binary"), reduce_order=1)
    f2w = scenes.cornell_camera(W, H)

    def oracle_render(p):
        diff.apply_params(rend.scene, mats, p)
        out, _ = ol.render(ol.SceneArrays(rend.scene.export()), st, SPP, W, H, f2w)
        return out

    t_oracle = oracle_render(scenes.perturbed_params(p0, mats, seed=2))
    pairs = [(0, 0), (0, 1), (2, 2), (4, 0), (6, 1), (15, 4), (15, 5)]
    g_fd = _fd(oracle_render, p0, t_oracle, pairs)
    # the adjoint against the oracle's own target and image
    img_o = oracle_render(p0)
    g_adj_o = rend.adjoint(p0, (2.0 * (img_o.astype(np.float64) - t_oracle)).astype(np.float32))
    a = np.array([g_adj_o[i, j] for i, j in pairs])
    err = _rel(a, g_fd)
    print(f"adjoint vs oracle FD rel err {err:.3e}")
    assert err <= 1e-2


def test_autograd_function_and_cost(lib):
    import torch
    rend, mats, p0, target = _setup()
    params = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    tgt = torch.from_numpy(target.astype(np.float32))
    t0 = time.perf_counter()
    img = diff.render(params, rend)
    t1 = time.perf_counter()
    loss = ((img - tgt) ** 2).sum()
    loss.backward()
    t2 = time.perf_counter()
    direct = rend.adjoint(p0, (2.0 * (img.detach().numpy().astype(np.float64) -
                                      target)).astype(np.float32))
    np.testing.assert_allclose(params.grad.numpy(), direct, rtol=1e-4, atol=1e-6)
    # cost: the adjoint (a forward render plus the replay) against a forward render
    r = rend.renderer
    fwd, adj = [], []
    for _ in range(5):
        rend.render(p0)
        fwd.append(r.stats()["kernel_ms"])
        rend.adjoint(p0, np.ones((H, W, 3), np.float32))
        adj.append(r.stats()["kernel_ms"])
    ratio = np.median(adj) / np.median(fwd)
    print(f"forward {np.median(fwd):.3f} ms, adjoint {np.median(adj):.3f} ms, ratio {ratio:.2f}; "
          f"autograd forward {1e3 * (t1 - t0):.1f} ms, backward {1e3 * (t2 - t1):.1f} ms")
    assert ratio <= 3.0
