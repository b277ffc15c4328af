"""GGX, the BSDF of the large-mesh and batched workloads, checked against its
published definition rather than against itself.

The reference has no microfacet BSDF (its glossy lobe is normalised Phong),
so GGX has no reference code to match.  Its oracle restatement and the
kernels' copy follow Walter, Marschner, Li and Torrance, "Microfacet Models
for Refraction through Rough Surfaces" (EGSR 2007): the GGX distribution D
(eq. 33), the separable Smith shadowing G1 of GGX (eq. 34), Schlick's
Fresnel term, and sampling of D(h)(n.h) (eqs. 35-36) with the sample weight
G (o.h) / ((o.n)(h.n)) times F.  These tests hold both to properties of that
definition that do not depend on how it is written:

* normalisation: the integral of D(h)(n.h) over the hemisphere is 1 (eq. 4
  of the paper), by quadrature, for alpha in {0.05, 0.2, 0.8};
* every sampled direction's weight equals eval(o, i) (n.i) / pdf(i) with
  pdf(i) = D(h)(n.h) / (4 (o.h)) (eq. 14 and the half-vector Jacobian);
* the mean sample weight (Monte Carlo over the draws) equals the quadrature
  of eval (n.i) over the hemisphere, within 3 standard errors;
* with F0 = 1 the directional albedo is at most 1 (no energy is created).

The CPU tests run them on the oracle; tests/test_gpu_parity.py runs them on
the kernels' code through path_debug_bsdf and also holds that code to the
oracle's bit for bit.
"""

import math

import numpy as np
import pytest

from path_gb300 import api
from oracle import oracle_lib as ol


def ggx(alpha, f0=0.04):
    return api.material("GGX", specular=(f0, f0, f0), roughness=alpha)


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _wo(theta_deg):
    """Direction towards the viewer at polar angle theta about n = +z; the
    BSDF takes the incoming ray direction, which is -wo."""
    t = math.radians(theta_deg)
    return np.array([math.sin(t), 0.0, math.cos(t)])


def normalisation(d_fn, alpha):
    """Integral of D(h)(n.h) over the hemisphere = 2 pi int_0^1 D(mu) mu dmu,
    by the trapezoid rule in s = log(1 - mu) (resolves the peak at mu = 1)."""
    s = np.linspace(math.log(1e-12), 0.0, 400001)
    x = np.exp(s)
    mu = 1.0 - x
    rec = np.zeros((len(mu), 9), np.float32)
    rec[:, 0] = mu
    rec[:, 1] = alpha
    d = d_fn(rec).astype(np.float64)
    f = d * mu * x  # dmu = -x ds
    head = 2 * math.pi * (1.0 / (math.pi * alpha * alpha)) * 1e-12  # mu in (1 - 1e-12, 1]
    trapezoid = float(np.sum((f[1:] + f[:-1]) * np.diff(s))) / 2
    return 2 * math.pi * trapezoid + head


def quadrature_albedo(eval_fn, theta_o, n_theta=1000, n_phi=1000):
    """int eval(o, i) (n.i) d omega_i over the hemisphere by the midpoint rule
    in (n.i, phi)."""
    wo = _wo(theta_o)
    c = (np.arange(n_theta) + 0.5) / n_theta
    p = (np.arange(n_phi) + 0.5) / n_phi * 2 * math.pi
    cc, pp = np.meshgrid(c, p, indexing="ij")
    sn = np.sqrt(1 - cc * cc)
    wi = np.stack([sn * np.cos(pp), sn * np.sin(pp), cc], -1).reshape(-1, 3)
    rec = np.zeros((len(wi), 9), np.float32)
    rec[:, 0:3] = -wo
    rec[:, 3:6] = wi
    rec[:, 8] = 1.0
    f = eval_fn(rec)[:, 0].astype(np.float64)
    return float(np.sum(f * cc.reshape(-1))) * (1.0 / n_theta) * (2 * math.pi / n_phi)


def sampled(sample_fn, theta_o, n=1 << 19, seed=0):
    rng = np.random.default_rng(seed)
    wo = _wo(theta_o)
    rec = np.zeros((n, 9), np.float32)
    rec[:, 0:3] = -wo
    rec[:, 5] = 1.0
    rec[:, 6:8] = rng.random((n, 2), dtype=np.float32)
    return rec, sample_fn(rec)


def check_normalisation(d_fn):
    for alpha in (0.05, 0.2, 0.8):
        assert abs(normalisation(d_fn, alpha) - 1.0) < 2e-4, alpha


def check_weights_match_eval_over_pdf(eval_fn, sample_fn, d_fn):
    for alpha in (0.05, 0.2, 0.8):
        for theta in (0.0, 35.0, 70.0):
            m = ggx(alpha)
            rec, out = sampled(lambda r: sample_fn(m, r), theta, n=20000, seed=1)
            w = out[:, 3].astype(np.float64)
            keep = w > 0
            wi = out[keep, 0:3].astype(np.float64)
            wo = np.broadcast_to(_wo(theta), wi.shape)
            h = _unit(wo + wi)
            ch = h[:, 2]
            oh = np.sum(wo * h, -1)
            drec = np.zeros((len(ch), 9), np.float32)
            drec[:, 0] = ch
            drec[:, 1] = alpha
            pdf = d_fn(drec).astype(np.float64) * ch / (4 * oh)
            erec = np.zeros((len(ch), 9), np.float32)
            erec[:, 0:3] = -wo
            erec[:, 3:6] = wi
            erec[:, 8] = 1.0
            f = eval_fn(m, erec)[:, 0].astype(np.float64)
            want = f * wi[:, 2] / pdf
            # float32 rounding of the direction and of both sides
            np.testing.assert_allclose(w[keep], want, rtol=2e-3, atol=1e-6)
            assert keep.mean() > 0.5


def check_mean_weight_is_albedo(eval_fn, sample_fn):
    for alpha in (0.2, 0.5, 0.8):
        for theta in (0.0, 45.0, 75.0):
            for f0 in (0.04, 1.0):
                m = ggx(alpha, f0)
                _, out = sampled(lambda r: sample_fn(m, r), theta, seed=2)
                w = out[:, 3].astype(np.float64)
                mc, se = w.mean(), w.std() / math.sqrt(len(w))
                quad = quadrature_albedo(lambda r: eval_fn(m, r), theta)
                assert abs(mc - quad) < 3 * se + 1e-3 * quad, (alpha, theta, f0, mc, quad, se)
                if f0 == 1.0:
                    assert mc <= 1.0 + 3 * se and quad <= 1.0 + 1e-3, (alpha, theta, mc, quad)


def _oracle_d(rec):
    return ol.debug_bsdf(ggx(0.1), 2, rec)


def test_ggx_distribution_is_normalised():
    check_normalisation(_oracle_d)


def test_ggx_sample_weights_are_eval_over_pdf():
    check_weights_match_eval_over_pdf(lambda m, r: ol.debug_bsdf(m, 0, r),
                                      lambda m, r: ol.debug_bsdf(m, 1, r), _oracle_d)


def test_ggx_mean_weight_is_the_directional_albedo():
    check_mean_weight_is_albedo(lambda m, r: ol.debug_bsdf(m, 0, r),
                                lambda m, r: ol.debug_bsdf(m, 1, r))


def test_ggx_is_reciprocal():
    # f(o, i) = f(i, o): D, G and F are symmetric in the two directions
    rng = np.random.default_rng(3)
    a = _unit(rng.normal(size=(5000, 3)))
    b = _unit(rng.normal(size=(5000, 3)))
    a[:, 2] = np.abs(a[:, 2])
    b[:, 2] = np.abs(b[:, 2])
    m = ggx(0.3, 0.5)
    r1 = np.zeros((5000, 9), np.float32)
    r1[:, 0:3] = -a
    r1[:, 3:6] = b
    r1[:, 8] = 1
    r2 = r1.copy()
    r2[:, 0:3] = -b
    r2[:, 3:6] = a
    np.testing.assert_allclose(ol.debug_bsdf(m, 0, r1), ol.debug_bsdf(m, 0, r2), rtol=2e-5)


if __name__ == "__main__":
    pytest.main([__file__, "-q"])
