"""Global-template fill: deterministic mode against the reference fixtures,
the atomic mode and itself (bit-identical on repeated runs)."""

import numpy as np
import pytest

from conftest import load_golden, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def dev(x):
    return torch.as_tensor(np.asarray(x), device="cuda")


def test_deterministic_fill_matches_reference():
    from gbgpu_gb300 import GBGPU
    g = load_golden("fill_basic")
    gb = GBGPU()
    t = dev(g["templates_before"]).clone()
    gb.fill_global_template(dev(g["group_index"]), t, dev(g["A"]), dev(g["E"]),
                            dev(g["start_inds"]), start_freq_ind=int(g["start_freq_ind"]),
                            mode="deterministic")
    t = t.cpu().numpy()
    np.testing.assert_array_equal(t[:, 2], g["templates_after"][:, 2])
    assert rel_err(t[:, :2], g["templates_after"][:, :2]) < 1e-13
    gen = torch.zeros(g["generated"].shape, dtype=torch.complex128, device="cuda")
    gb.generate_global_template(g["params"].T, dev(g["group_index"]), gen, N=int(g["N"]),
                                T=float(g["T"]), dt=float(g["dt"]),
                                start_freq_ind=int(g["start_freq_ind"]), fill_mode="deterministic")
    assert rel_err(gen.cpu().numpy(), g["generated"]) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_deterministic_fill_is_bit_reproducible_and_matches_atomic(precision):
    from gbgpu_gb300 import GBGPU
    rng = np.random.default_rng(90)
    B, G, N = 6000, 5, 256
    T, dt = 4 * 31557600.0, 10.0
    # a dense band: hundreds of windows overlap every covered bin of a group
    f0 = rng.uniform(1.0e-3, 1.002e-3, B)
    fdot = 10 ** rng.uniform(-18, -16, B)
    p = np.array([10 ** rng.uniform(-23, -21, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B))])
    gi = dev(rng.integers(0, G, B).astype(np.int32))
    s0 = int(1.0e-3 * T) - 400
    L = 2000
    gb = GBGPU()
    out = []
    for mode in ("deterministic", "deterministic", "atomic"):
        t = torch.full((G, 2, L), 7.0 + 1j, dtype=torch.complex128, device="cuda")
        gb.generate_global_template(p.T, gi, t, N=N, T=T, dt=dt, start_freq_ind=s0,
                                    precision=precision, fill_mode=mode)
        out.append(t.cpu().numpy())
    np.testing.assert_array_equal(out[0], out[1])
    # mixed: the deterministic path forms A/E from the FP64-scaled X/Y/Z, the
    # fused atomic path in FP32 before scaling -- FP32-level differences
    assert rel_err(out[0], out[2]) < (1e-13 if precision == "fp64" else 1e-6)
    # the windows cover ~500 of the 2000 bins of each group; the rest is 0
    assert 0.2 * out[0].size < np.count_nonzero(out[0]) < 0.3 * out[0].size


@pytest.mark.parametrize("precision,N", [("fp64", 256), ("mixed", 256), ("mixed", 64),
                                         ("pair", 256), ("pair", 64)])
def test_sorted_fill_prereduces_and_matches(precision, N):
    """Binaries launched in (group, carrier bin) order: the fused fill adds each
    tile's overlapping same-group windows once per output bin.  Same templates
    as the unsorted launch and the deterministic gather (FP64 rounding of the
    summation order only); a group boundary and windows past both ends of the
    data inside one tile; windows of invalid (out-of-range group) binaries
    are dropped and flagged."""
    from gbgpu_gb300 import GBGPU
    rng = np.random.default_rng(91 + N)
    B, G = 3000, 3
    T, dt = 4 * 31557600.0, 10.0
    f0 = rng.uniform(1.0e-3, 1.001e-3, B)
    fdot = 10 ** rng.uniform(-18, -16, B)
    p = np.array([10 ** rng.uniform(-23, -21, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B))])
    gi = rng.integers(0, G, B).astype(np.int32)
    q = np.rint(f0 * T)
    s0 = int(q.min()) + 20                  # the lowest windows start before bin 0
    L = int(q.max()) - s0 - 10              # and the highest end past the last bin
    gb = GBGPU()
    out = {}
    for key, mode, sort in (("unsorted", "atomic", False), ("sorted", "atomic", True),
                            ("det", "deterministic", False)):
        t = torch.zeros((G, 2, L), dtype=torch.complex128, device="cuda")
        gb.generate_global_template(p.T, dev(gi), t, N=N, T=T, dt=dt, start_freq_ind=s0,
                                    precision=precision, fill_mode=mode, sort=sort)
        out[key] = t.cpu().numpy()
    scale = np.max(np.abs(out["det"]))
    assert np.max(np.abs(out["sorted"] - out["unsorted"])) <= 1e-12 * scale
    if precision == "fp64":
        assert np.max(np.abs(out["sorted"] - out["det"])) <= 1e-12 * scale
    if precision == "pair":
        # the pair form's fill against the FP64 form's gather (1e-10 per window)
        t = torch.zeros((G, 2, L), dtype=torch.complex128, device="cuda")
        gb.generate_global_template(p.T, dev(gi), t, N=N, T=T, dt=dt, start_freq_ind=s0,
                                    precision="fp64", fill_mode="deterministic")
        ref = t.cpu().numpy()
        assert np.max(np.abs(out["unsorted"] - ref)) <= 1e-10 * np.max(np.abs(ref))
    # add_to_templates with the same option, on top of the sorted result
    tA = torch.as_tensor(out["sorted"][:, 0].copy(), device="cuda")
    tE = torch.as_tensor(out["sorted"][:, 1].copy(), device="cuda")
    gb.add_to_templates(torch.as_tensor(p, device="cuda"), dev(gi), (tA, tE), N=N, T=T, dt=dt,
                        start_freq_ind=s0, precision=precision, sort=True)
    assert np.max(np.abs(tA.cpu().numpy() - 2 * out["sorted"][:, 0])) <= 2e-12 * scale
    # an out-of-range group drops that binary's window and raises on the status
    bad = gi.copy()
    bad[5] = G + 3
    t = torch.zeros((G, 2, L), dtype=torch.complex128, device="cuda")
    with pytest.raises(ValueError):
        gb.generate_global_template(p.T, dev(bad), t, N=N, T=T, dt=dt, start_freq_ind=s0,
                                    precision=precision, sort=True)
