"""Host-side helpers of bench.py (CPU): the EPL term count it reports and the
algorithmic flop count its roofline divides by."""
import numpy as np
import pytest
import torch

import bench
from gigalens_gb300 import workloads as W
from oracle import lens_oracle as O


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_epl_terms_matches_the_oracle_rule(seed):
    xs = W.draw_params(4096, seed=seed)[0][0]
    e1, e2 = xs["e1"].numpy(), xs["e2"].numpy()
    assert bench.epl_terms(e1, e2) == O.epl_term_count(torch.tensor(e1), torch.tensor(e2), 50)


def test_epl_terms_round_lens_and_cap():
    # f = 0: niter = log(1e-12) / log(0) + 2 = 2, one iteration (i = 1 < 2)
    assert bench.epl_terms(np.zeros(4), np.zeros(4)) == 1
    assert bench.epl_terms(np.array([0.6]), np.array([0.6]), cap=50) == 50


def test_flop_count_of_the_headline_workload():
    """90x90 px, ss = 2, 41x41 supersampled PSF, K = 31: 95.6 MFLOP per
    likelihood + gradient evaluation (forward 31.9 M + adjoint 63.7 M)."""
    fwd, adj = bench.flops_per_eval(31)
    assert fwd + adj == 95_644_800
    Ps, P = 180 * 180, 90 * 90
    assert fwd == Ps * (84 + 310) + 2 * P * 42 ** 2 + 12 * P
    assert adj - fwd == Ps * (84 + 310)


def test_flop_count_of_the_least_squares_workload():
    """100x100 px, ss = 2, 21x21 supersampled PSF (22x22 combined kernel),
    45 shapelet channels: basis 110 per supersampled pixel, 45 strided
    correlations, A^T W A counted once, A^T W b."""
    f = bench.lstsq_flops(100)
    P = 100 * 100
    assert f["basis"] == 110 * 200 * 200
    assert f["psf"] == 45 * 2 * P * 22 ** 2
    assert f["gram"] == 2 * P * 45 * 46 / 2
    assert f["rhs"] == 2 * P * 45
    assert sum(f.values()) == 461_600_000
