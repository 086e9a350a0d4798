"""R-hat and cross-chain ESS on chains with known answers (CPU)."""
import numpy as np
import torch

from gigalens_gb300.cuda.diagnostics import effective_sample_size, potential_scale_reduction


def test_rhat_iid_and_shifted():
    g = torch.Generator().manual_seed(0)
    x = torch.randn(2000, 8, 3, generator=g)
    r = potential_scale_reduction(x)
    assert (r - 1).abs().max() < 0.01
    x[:, 0] += 3.0          # one chain off: R-hat well above 1
    assert potential_scale_reduction(x)[0] > 1.1


def test_ess_iid_and_ar1():
    g = torch.Generator().manual_seed(1)
    n, m = 4000, 8
    x = torch.randn(n, m, 2, generator=g, dtype=torch.float64)
    ess = effective_sample_size(x)
    assert ((ess / (n * m)) - 1).abs().max() < 0.15
    # AR(1) with coefficient phi: ESS ~ n m (1 - phi) / (1 + phi)
    phi = 0.8
    e = torch.randn(n, m, generator=g, dtype=torch.float64)
    y = torch.zeros(n, m, dtype=torch.float64)
    for t in range(1, n):
        y[t] = phi * y[t - 1] + e[t]
    ess = float(effective_sample_size(y[:, :, None])[0])
    expect = n * m * (1 - phi) / (1 + phi)
    assert 0.75 * expect < ess < 1.25 * expect


def test_dual_averaging_reductions():
    """The step-size adaptation's reduction over chains: the log-harmonic mean
    (TFP's default) follows the least-accepting chain, the mean does not."""
    import math

    from gigalens_gb300.cuda.inference import _DualAveraging

    la = torch.full((2048,), math.log(0.99))
    la[0] = math.log(1e-4)                       # one chain that rejects
    steps = {}
    for reduce in ("harmonic", "mean"):
        da = _DualAveraging(0.3, 0.75, torch.device("cpu"), reduce=reduce)
        for _ in range(20):
            da.update(la)
        steps[reduce] = float(da.step_size[0])
    assert steps["harmonic"] < 0.3 < steps["mean"]
