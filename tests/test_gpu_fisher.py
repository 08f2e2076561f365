"""Batched per-binary Fisher matrices (GBGPUBase.fisher_matrices).

Checked against the exact FP64 Fisher matrix of the torch restatement
(oracle/fastgb_torch.py): J_i = dh/dtheta_i by forward mode, F_ij = 4/T
sum Re conj(J_i) J_j / S over the A, E windows, within 1e-5 of
sqrt(F_ii F_jj) for the five-point differences (measured worst 3.2e-6) and
within 2e-6 for the in-kernel forward mode (gbx_fisher; measured worst
3.6e-7, its FP32 tangents).  Includes binaries whose f0 sits next to a bin
boundary (the difference stencil moves their window), TDI-2 and the
third-body model (differences only).
"""

import numpy as np
import pytest

import fastgb_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0
DT = 10.0


def _exact_fisher(p, th, N, tdi2=False):
    import fastgb_torch as FT
    from gbgpu_gb300.sensitivity import A1TDISens
    Tu = int(T_OBS / DT) * DT
    pt = torch.as_tensor(p)
    tt = None if th is None else torch.as_tensor(th)
    rows = p.shape[0] + (0 if th is None else th.shape[0])
    J = []
    for k in range(rows):
        dp = torch.zeros_like(pt)
        dt_ = None if tt is None else torch.zeros_like(tt)
        if k < p.shape[0]:
            dp[k] = 1.0
        else:
            dt_[k - p.shape[0]] = 1.0
        if tt is None:
            _, j = torch.func.jvp(lambda x: FT.waveform_aet(x, N, T_OBS, DT, tdi2=tdi2), (pt,), (dp,))
        else:
            _, j = torch.func.jvp(lambda x, y: FT.waveform_aet(x, N, T_OBS, DT, third=y),
                                  (pt, tt), (dp, dt_))
        J.append(j.numpy())
    J = np.stack(J, 1)                                   # (B, n, 2, N)
    start = O.start_indices(p[1], N, T_OBS, DT)
    S = A1TDISens.get_Sn((start[:, None] + np.arange(N)[None, :]) / Tu)
    return 4.0 / Tu * np.einsum("bicn,bjcn->bij", np.conj(J) / S[:, None, None, :], J).real


@pytest.mark.parametrize("third,method,N,tdi2", [(False, "differences", 256, False),
                                                 (False, "forward", 256, False),
                                                 (False, "forward", 128, True),
                                                 (False, "forward", 1024, False),
                                                 (True, "differences", 256, False)])
def test_fisher_matrices_match_exact_forward_mode(third, method, N, tdi2):
    from gbgpu_gb300 import GBGPU, GBGPUThirdBody
    rng = np.random.default_rng(9 + N)
    B = 12
    Tu = int(T_OBS / DT) * DT
    q = np.rint(rng.uniform(2e-3, 4e-3, B) * Tu)
    frac = rng.uniform(-0.3, 0.3, B)
    frac[:3] = [0.49995, -0.49995, 0.4999]                 # stencil crosses a bin edge
    f0 = (q + frac) / Tu
    fdot = 10 ** rng.uniform(-17, -16, B)
    p = np.array([10 ** rng.uniform(-22.3, -21.7, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0.5, 5.5, B), np.arccos(rng.uniform(-0.9, 0.9, B)),
                  rng.uniform(0.3, 2.8, B), rng.uniform(0.5, 5.5, B),
                  np.arcsin(rng.uniform(-0.9, 0.9, B))])
    th = None
    if third:
        P2 = 10 ** rng.uniform(0.3, 1.0, B)
        th = np.array([10 ** rng.uniform(0.5, 1.5, B), rng.uniform(0.3, 6.0, B),
                       rng.uniform(0.1, 0.8, B), P2, rng.uniform(0.1, 0.9, B) * P2])
    gb = GBGPUThirdBody() if third else GBGPU()
    full = p if th is None else np.concatenate([p, th])
    F = gb.fisher_matrices(full, N=N, T=T_OBS, dt=DT, tdi2=tdi2, method=method)
    ref = _exact_fisher(p, th, N, tdi2)
    d = np.sqrt(np.einsum("bii->bi", ref))
    err = np.abs(F - ref) / (d[:, :, None] * d[:, None, :])
    print(f"{method} N={N} tdi2={tdi2} third={third}: max |F - F_exact| / sqrt(F_ii F_jj) = "
          f"{err.max():.2e}")
    tol = {"forward": 2e-6, "differences": 1e-5}[method]
    assert np.max(err) < tol, np.unravel_index(np.argmax(err), err.shape)


def test_forward_fisher_matches_differences_on_a_batch():
    """Uneven sky positions and frequencies across 2e-4..2e-2 Hz, inds subset;
    the bound is the differences' own (measured worst 4.5e-6)."""
    from gbgpu_gb300 import GBGPU
    rng = np.random.default_rng(31)
    B, N = 300, 512
    Tu = int(T_OBS / DT) * DT
    q = np.rint(10 ** rng.uniform(np.log10(2e-4), np.log10(2e-2), B) * Tu)
    f0 = (q + rng.uniform(-0.3, 0.3, B)) / Tu
    fdot = 10 ** rng.uniform(-18, -15.5, B)
    p = np.array([10 ** rng.uniform(-23, -21, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B))])
    gb = GBGPU()
    inds = [0, 1, 2, 4, 5, 6, 7, 8]
    Ff = gb.fisher_matrices(p, N=N, T=T_OBS, dt=DT, tdi2=True, inds=inds, method="forward")
    Fd = gb.fisher_matrices(p, N=N, T=T_OBS, dt=DT, tdi2=True, inds=inds, method="differences")
    d = np.sqrt(np.einsum("bii->bi", Fd))
    err = np.abs(Ff - Fd) / (d[:, :, None] * d[:, None, :])
    print(f"forward vs differences, {B} binaries: max normalised difference {err.max():.2e}")
    assert np.max(err) < 1e-5


def test_forward_fisher_declines_the_third_body():
    from gbgpu_gb300 import GBGPUThirdBody
    p = np.zeros((14, 2))
    with pytest.raises(ValueError, match="9-parameter"):
        GBGPUThirdBody().fisher_matrices(p, N=256, method="forward")


def test_information_matrix_forward_mode_is_the_log_parameter_fisher():
    """The reference's information_matrix differentiates with relative steps,
    so its matrices are in ln theta; the forward-mode path equals the exact
    Fisher matrix scaled by theta_i theta_j (2e-6 of sqrt(F_ii F_jj)) and the
    reference's differences to their own noise (eps = 1e-9 relative steps
    leave ~1e-3)."""
    from gbgpu_gb300 import GBGPU
    rng = np.random.default_rng(19)
    B, N = 8, 256
    Tu = int(T_OBS / DT) * DT
    q = np.rint(rng.uniform(2e-3, 4e-3, B) * Tu)
    f0 = (q + rng.uniform(-0.3, 0.3, B)) / Tu
    fdot = 10 ** rng.uniform(-17, -16, B)
    p = np.array([10 ** rng.uniform(-22.3, -21.7, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0.5, 5.5, B), np.arccos(rng.uniform(-0.9, 0.9, B)),
                  rng.uniform(0.3, 2.8, B), rng.uniform(0.5, 5.5, B),
                  np.arcsin(rng.uniform(-0.9, 0.9, B))])
    inds = [0, 1, 2, 4, 5, 6, 7, 8]
    gb = GBGPU()
    Ff = gb.information_matrix(p.copy(), inds=inds, N=N, T=T_OBS, dt=DT, method="forward")
    ref = _exact_fisher(p, None, N) * p.T[:, :, None] * p.T[:, None, :]
    ref = ref[:, inds][:, :, inds]
    d = np.sqrt(np.einsum("bii->bi", ref))
    err = np.abs(Ff - ref) / (d[:, :, None] * d[:, None, :])
    print(f"information_matrix forward vs exact: {err.max():.2e}")
    assert err.max() < 2e-6
    # the reference's differences require one start bin per call: one binary each
    Fd = np.concatenate([gb.information_matrix(p[:, b:b + 1].copy(), inds=inds, N=N, T=T_OBS,
                                               dt=DT, method="differences") for b in range(B)])
    errd = np.abs(Fd - ref) / (d[:, :, None] * d[:, None, :])
    print(f"information_matrix differences vs exact: {errd.max():.2e}")
    assert errd.max() < 1e-2


def test_information_matrix_forward_mode_with_parameter_transforms():
    """Sampled coordinates ln amp, cos iota, sin beta (the reference's
    parameter_transforms): the forward path runs the kernel at the physical
    parameters and applies D = theta_l dphi_k/dtheta_l, so it equals
    D^T F_exact D of the exact FP64 Fisher matrix (2e-6 of sqrt(F_ii F_jj))
    and the reference's differences to their own noise."""
    from gbgpu_gb300 import GBGPU
    rng = np.random.default_rng(23)
    B, N = 6, 256
    Tu = int(T_OBS / DT) * DT
    q = np.rint(rng.uniform(2e-3, 4e-3, B) * Tu)
    f0 = (q + rng.uniform(-0.3, 0.3, B)) / Tu
    fdot = 10 ** rng.uniform(-17, -16, B)
    phys = np.array([10 ** rng.uniform(-22.3, -21.7, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                     rng.uniform(0.5, 5.5, B), np.arccos(rng.uniform(-0.9, 0.9, B)),
                     rng.uniform(0.3, 2.8, B), rng.uniform(0.5, 5.5, B),
                     np.arcsin(rng.uniform(-0.9, 0.9, B))])
    th = phys.copy()
    th[0], th[5], th[8] = np.log(phys[0]), np.cos(phys[5]), np.sin(phys[8])
    tr = {0: np.exp, 5: np.arccos, 8: np.arcsin}
    inds = [0, 1, 2, 4, 5, 6, 7, 8]
    gb = GBGPU()
    Ff = gb.information_matrix(th.copy(), inds=inds, N=N, T=T_OBS, dt=DT,
                               parameter_transforms=tr, method="forward")
    D = np.zeros((B, 9, 9))
    for b in range(B):
        D[b] = np.diag(th[:, b])
        D[b, 0, 0] = th[0, b] * phys[0, b]                       # d exp(x) = exp(x) dx
        D[b, 5, 5] = -th[5, b] / np.sqrt(1 - th[5, b] ** 2)      # d arccos(x)
        D[b, 8, 8] = th[8, b] / np.sqrt(1 - th[8, b] ** 2)       # d arcsin(x)
    ref = np.einsum("bki,bkl,blj->bij", D, _exact_fisher(phys, None, N), D)[:, inds][:, :, inds]
    d = np.sqrt(np.einsum("bii->bi", ref))
    err = np.abs(Ff - ref) / (d[:, :, None] * d[:, None, :])
    print(f"information_matrix forward with transforms vs exact: {err.max():.2e}")
    assert err.max() < 2e-6
    Fd = np.concatenate([gb.information_matrix(th[:, b:b + 1].copy(), inds=inds, N=N, T=T_OBS,
                                               dt=DT, parameter_transforms=tr,
                                               method="differences") for b in range(B)])
    errd = np.abs(Fd - ref) / (d[:, :, None] * d[:, None, :])
    print(f"information_matrix differences with transforms vs exact: {errd.max():.2e}")
    assert errd.max() < 1e-2
