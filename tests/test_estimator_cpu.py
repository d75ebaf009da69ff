"""The learned estimator's oracle and host interface, on the CPU.

* The NumPy oracle's gradients (oracle/estimator_oracle.py) equal central finite differences of its
  own loss (BF16 rounding off), for parameters of every layer: its backward pass is the derivative
  of its forward pass.
* The parameter vector's layout matches the size the library reports.
"""
from __future__ import annotations

import numpy as np


def test_parameter_count(am):
    from oracle import estimator_oracle as eo
    assert am.Estimator.param_count() == sum(int(np.prod(s)) for _, s in eo.SIZES) == 41313


def test_oracle_gradients_match_finite_differences():
    from oracle import estimator_oracle as eo
    rng = np.random.default_rng(3)
    p = {}
    for name, shape in eo.SIZES:
        p[name] = rng.normal(0, 0.3 if name.startswith("W") else 0.1, shape)
    p["W1"][81:] = 0.0
    params = eo.pack(p)
    x = rng.normal(0, 1, (3, 3, 512))
    t = rng.normal(0, 1, 3)
    eo.EXACT = True
    try:
        g, _ = eo.gradients(params, x, t)
        names = [n for n, _ in eo.SIZES]
        offs = np.cumsum([0] + [int(np.prod(s)) for _, s in eo.SIZES])
        for li, name in enumerate(names):
            for j in rng.choice(offs[li + 1] - offs[li], min(3, offs[li + 1] - offs[li]), replace=False):
                k = offs[li] + j
                if name == "W1" and j // 16 >= 81:
                    continue
                e = 1e-6
                pp, pm = params.copy(), params.copy()
                pp[k] += e
                pm[k] -= e
                _, lp = eo.gradients(pp, x, t)
                _, lm = eo.gradients(pm, x, t)
                fd = (lp - lm) / (2 * e)
                assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), f"{name}[{j}]: {g[k]} vs {fd}"
    finally:
        eo.EXACT = False
