"""MCMC diagnostics used with the HMC chains (``tf-demo.ipynb`` cell 18:
``tfp.mcmc.potential_scale_reduction`` and ``tfp.mcmc.effective_sample_size``
with ``cross_chain_dims=1``), restated in PyTorch.

Conventions follow TFP's documentation: samples are ``(n_results, n_chains, ...)``.

* R-hat (not split): with n draws per chain, W the mean within-chain
  variance (ddof 1) and B/n the variance of the chain means (ddof 1),
  sigma2+ = (n-1)/n W + B/n and R-hat = (m+1)/m sigma2+/W - (n-1)/(m n),
  m chains (Brooks & Gelman 1998, as in TFP).
* ESS across chains (Gelman et al., BDA3 sec. 11.5): the autocorrelation at
  lag t is rho_t = 1 - (W - mean_chains(autocov_t)) / sigma2+, summed in
  pairs while the pair sums stay positive (Geyer's initial positive
  sequence); ESS = m n / (-1 + 2 sum rho).
"""
import torch


def potential_scale_reduction(samples: torch.Tensor) -> torch.Tensor:
    x = samples.double()
    n, m = x.shape[0], x.shape[1]
    means = x.mean(0)
    W = x.var(0, unbiased=True).mean(0)
    B_over_n = means.var(0, unbiased=True)
    sigma2 = (n - 1) / n * W + B_over_n
    return ((m + 1) / m * sigma2 / W - (n - 1) / (m * n)).to(samples.dtype)


def _autocov(x: torch.Tensor) -> torch.Tensor:
    """Autocovariance along dim 0 via FFT (biased, divided by n)."""
    n = x.shape[0]
    xc = x - x.mean(0, keepdim=True)
    L = 1
    while L < 2 * n:
        L *= 2
    f = torch.fft.rfft(xc, n=L, dim=0)
    ac = torch.fft.irfft(f * f.conj(), n=L, dim=0)[:n]
    return ac / n


def effective_sample_size(samples: torch.Tensor, cross_chain_dims=1) -> torch.Tensor:
    x = samples.double()
    n, m = x.shape[0], x.shape[1]
    acov = _autocov(x)                         # (n, m, ...)
    W = x.var(0, unbiased=True).mean(0)
    B_over_n = x.mean(0).var(0, unbiased=True) if m > 1 else torch.zeros_like(W)
    sigma2 = (n - 1) / n * W + B_over_n
    # unbiased within-chain autocovariance scale, BDA3 11.7
    rho = 1.0 - (W - acov.mean(1) * n / (n - 1)) / sigma2   # (n, ...)
    rho[0] = 1.0
    # Geyer initial positive sequence over pairs (rho_{2k} + rho_{2k+1})
    npairs = n // 2
    pairs = rho[: 2 * npairs].reshape(npairs, 2, *rho.shape[1:]).sum(1)
    positive = pairs > 0
    mask = torch.cumprod(positive.to(torch.int64), dim=0).to(rho.dtype)
    tau = -1.0 + 2.0 * (pairs * mask).sum(0)
    return (m * n / tau).to(samples.dtype)
