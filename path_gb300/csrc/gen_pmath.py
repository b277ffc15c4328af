"""Fit the polynomial coefficients used by ``pmath.h``.

The renderer's single-precision transcendental functions (sin, cos, asin,
acos; pow is evaluated in double precision by pmath.h itself) are evaluated by our own polynomial approximations so that the CUDA kernels
and the CPU oracle produce the same bits: both sides run the same sequence of
IEEE-754 single-precision multiplies, adds, divides and square roots, with no
fused multiply-add.  The coefficients come from a weighted least-squares fit
on Chebyshev nodes followed by Lawson iterations (an iteratively reweighted
least-squares route to the minimax polynomial), done in float64 and rounded
to float32.

Run ``python gen_pmath.py`` to rewrite ``pmath_coeffs.h``; it also prints the
worst error, in float32 ulps, of each function evaluated exactly as
``pmath.h`` evaluates it (emulated with numpy float32 arithmetic).
"""

import os

import numpy as np


def _fit(target, lo, hi, degree, basis, weight, n=4000, lawson_iters=60):
    """Minimax-style fit of ``target(z) ~ sum c_k basis(z)**k`` on [lo, hi]."""
    k = np.arange(n)
    z = 0.5 * (lo + hi) + 0.5 * (hi - lo) * np.cos(np.pi * (k + 0.5) / n)
    y = target(z)
    w_rel = weight(z)
    a = np.stack([basis(z) ** i for i in range(degree + 1)], axis=1)
    lw = np.ones(n) / n
    coef = None
    for _ in range(lawson_iters):
        sw = np.sqrt(lw) * w_rel
        coef, *_ = np.linalg.lstsq(a * sw[:, None], y * sw, rcond=None)
        err = np.abs((a @ coef - y) * w_rel)
        lw = lw * (err + 1e-300)
        lw /= lw.sum()
    return coef


def _horner32(coefs, x):
    x = np.float32(x) if np.isscalar(x) else x.astype(np.float32)
    acc = np.full_like(x, np.float32(coefs[-1]), dtype=np.float32)
    for c in coefs[-2::-1]:
        acc = (acc * x).astype(np.float32)
        acc = (acc + np.float32(c)).astype(np.float32)
    return acc


def fit_all():
    out = {}
    # sin(r) = r + r^3 * S(r^2),  |r| <= pi/4
    lim = (np.pi / 4) ** 2
    s = _fit(lambda u: (np.sin(np.sqrt(u)) - np.sqrt(u)) / (u * np.sqrt(u)),
             1e-12, lim, 4, lambda u: u, lambda u: u * np.sqrt(u) / np.sin(np.sqrt(u)))
    out["SIN"] = s
    # cos(r) = 1 - r^2/2 + r^4 * C(r^2)
    c = _fit(lambda u: (np.cos(np.sqrt(u)) - 1 + u / 2) / (u * u),
             1e-12, lim, 4, lambda u: u, lambda u: u * u / np.cos(np.sqrt(u)))
    out["COS"] = c
    # asin(x) = x + x^3 * A(x^2),  |x| <= 0.5
    a = _fit(lambda u: (np.arcsin(np.sqrt(u)) - np.sqrt(u)) / (u * np.sqrt(u)),
             1e-12, 0.25, 6, lambda u: u,
             lambda u: u * np.sqrt(u) / np.arcsin(np.sqrt(u)))
    out["ASIN"] = a
    return out


def _ulps(approx, exact):
    exact32 = exact.astype(np.float32)
    spacing = np.spacing(np.abs(exact32)).astype(np.float64)
    return np.max(np.abs(approx.astype(np.float64) - exact) / spacing)


def report(coefs):
    c32 = {k: [np.float32(v) for v in vals] for k, vals in coefs.items()}
    r = np.linspace(-np.pi / 4, np.pi / 4, 200001).astype(np.float32)
    r2 = (r * r).astype(np.float32)
    sin_a = (r + (r * r2).astype(np.float32) * _horner32(c32["SIN"], r2)).astype(np.float32)
    half = (np.float32(0.5) * r2).astype(np.float32)
    cos_a = ((np.float32(1) - half).astype(np.float32)
             + ((r2 * r2).astype(np.float32) * _horner32(c32["COS"], r2)).astype(np.float32)
             ).astype(np.float32)
    print("sin ulps", _ulps(sin_a[r != 0], np.sin(r[r != 0].astype(np.float64))))
    print("cos ulps", _ulps(cos_a, np.cos(r.astype(np.float64))))
    x = np.linspace(0, 0.5, 200001).astype(np.float32)[1:]
    x2 = (x * x).astype(np.float32)
    as_a = (x + (x * x2).astype(np.float32) * _horner32(c32["ASIN"], x2)).astype(np.float32)
    print("asin ulps", _ulps(as_a, np.arcsin(x.astype(np.float64))))


def write_header(coefs, path):
    lines = [
        "// Generated by gen_pmath.py: polynomial coefficients for pmath.h.",
        "// Each array lists coefficients from the constant term upwards.",
        "#pragma once",
        "",
    ]
    for name, vals in coefs.items():
        body = ", ".join(f"{np.float32(v).item():.9e}f" for v in vals)
        lines.append(f"#define PM_{name}_DEGREE {len(vals) - 1}")
        lines.append(f"#define PM_{name}_COEFFS {{{body}}}")
        lines.append("")
    with open(path, "w") as fh:
        fh.write("\n".join(lines))


if __name__ == "__main__":
    cf = fit_all()
    report(cf)
    write_header(cf, os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                  "pmath_coeffs.h"))
