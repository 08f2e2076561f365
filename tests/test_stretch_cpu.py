"""Stretch-move ensemble update (gbgpu_gb300.mcmc.stretch_update) on CPU.

The GPU sampler (StretchSampler) calls the same update with the fused
likelihood; here it samples known targets with a plain torch log-density:
three independent correlated Gaussians in 4-D (one per ensemble), whose means
and covariances the chains must recover, a bounded target whose walkers must
never leave the box, and the stretch factors' distribution g(z) ~ 1/sqrt(z).
"""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gbgpu_gb300.mcmc import stretch_draws, stretch_update, stretch_z  # noqa: E402


def test_stretch_z_distribution():
    a = 2.0
    u = torch.rand(200_000, generator=torch.Generator().manual_seed(1), dtype=torch.float64)
    z = stretch_z(u, a)
    assert float(z.min()) >= 1 / a and float(z.max()) <= a
    # CDF of g(z) ~ 1/sqrt(z) on [1/a, a]: (sqrt(z) - 1/sqrt(a)) / (sqrt(a) - 1/sqrt(a))
    zs = np.sort(z.numpy())
    cdf = (np.sqrt(zs) - 1 / np.sqrt(a)) / (np.sqrt(a) - 1 / np.sqrt(a))
    ks = np.max(np.abs(cdf - (np.arange(zs.size) + 0.5) / zs.size))
    assert ks < 0.005


def _gaussians(B, d, seed):
    rng = np.random.default_rng(seed)
    mus, covs = [], []
    for _ in range(B):
        A = rng.standard_normal((d, d))
        cov = A @ A.T + 0.3 * np.eye(d)
        covs.append(cov)
        mus.append(rng.standard_normal(d) * 3)
    return np.array(mus), np.array(covs)


def test_stretch_recovers_gaussian_moments():
    B, d, W, steps, burn = 3, 4, 32, 3000, 500
    mus, covs = _gaussians(B, d, 11)
    mu_t = torch.as_tensor(mus)                                # (B, d)
    P_t = torch.as_tensor(np.linalg.inv(covs))                 # (B, d, d)

    def loglike(Y):                                            # (d, B, Wh) -> (B, Wh)
        r = Y.permute(1, 2, 0) - mu_t[:, None, :]
        return -0.5 * torch.einsum("bwi,bij,bwj->bw", r, P_t, r)

    g = torch.Generator().manual_seed(5)
    x = (mu_t.T[:, :, None] + 0.1 * torch.randn((d, B, W), generator=g, dtype=torch.float64))
    x = x.contiguous()
    logL = torch.cat([loglike(x[:, :, :W // 2]), loglike(x[:, :, W // 2:])], 1)
    acc = torch.zeros((B, W), dtype=torch.int64)
    free = torch.arange(d)
    u, j, lu = stretch_draws(steps, B, W // 2, g, "cpu")
    samples = []
    for s in range(steps):
        for h in (0, 1):
            stretch_update(x, logL, acc, h, u[s, h], j[s, h], lu[s, h], loglike, free)
        if s >= burn:
            samples.append(x.clone())
    # the cached log-likelihoods are those of the current walkers
    torch.testing.assert_close(logL, torch.cat([loglike(x[:, :, :W // 2]),
                                                loglike(x[:, :, W // 2:])], 1))
    S = torch.stack(samples)                                   # (n, d, B, W)
    frac = acc.sum().item() / (B * W * steps)
    assert 0.2 < frac < 0.9
    for b in range(B):
        pts = S[:, :, b, :].permute(0, 2, 1).reshape(-1, d).numpy()
        sd = np.sqrt(np.diag(covs[b]))
        # means within 0.15 sigma, covariances within 15 % (of the variances' scale)
        assert np.all(np.abs(pts.mean(0) - mus[b]) < 0.15 * sd)
        emp = np.cov(pts.T)
        scale = np.sqrt(np.outer(np.diag(covs[b]), np.diag(covs[b])))
        assert np.all(np.abs(emp - covs[b]) < 0.15 * scale)


def test_stretch_bounds_are_respected():
    B, d, W, steps = 2, 2, 16, 400
    lo, hi = -1.0, 1.0

    def loglike(Y):                                            # flat inside: walkers fill the box
        return torch.zeros(Y.shape[1:], dtype=Y.dtype)

    g = torch.Generator().manual_seed(9)
    x = (0.2 * torch.rand((d, B, W), generator=g, dtype=torch.float64) - 0.1).contiguous()
    logL = torch.zeros((B, W), dtype=torch.float64)
    acc = torch.zeros((B, W), dtype=torch.int64)
    bounds = torch.tensor([[lo, hi]] * d, dtype=torch.float64)
    u, j, lu = stretch_draws(steps, B, W // 2, g, "cpu")
    for s in range(steps):
        for h in (0, 1):
            stretch_update(x, logL, acc, h, u[s, h], j[s, h], lu[s, h], loglike,
                           torch.arange(d), bounds=bounds)
        assert float(x.min()) >= lo and float(x.max()) <= hi
    # the walkers spread over the box (the ensemble starts in a 0.2-wide ball)
    assert float(x.std()) > 0.3
    assert 0 < acc.sum().item() < B * W * steps


def test_stretch_update_moves_only_free_coordinates():
    d, B, W = 3, 2, 8
    g = torch.Generator().manual_seed(3)
    x = torch.randn((d, B, W), generator=g, dtype=torch.float64).contiguous()
    fixed = x[1].clone()
    logL = torch.zeros((B, W), dtype=torch.float64)
    acc = torch.zeros((B, W), dtype=torch.int64)
    u, j, _ = stretch_draws(1, B, W // 2, g, "cpu")
    always = torch.full((B, W // 2), -math.inf, dtype=torch.float64)     # accept every move
    stretch_update(x, logL, acc, 0, u[0, 0], j[0, 0], always,
                   lambda Y: torch.zeros(Y.shape[1:], dtype=Y.dtype), torch.tensor([0, 2]))
    assert torch.equal(x[1], fixed)
    assert int(acc[:, :W // 2].sum()) == B * W // 2 and int(acc[:, W // 2:].sum()) == 0
