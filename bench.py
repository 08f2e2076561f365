"""Throughput of the FastGB hot path on GB300: fused waveform + log-likelihood.

Workload (one step = one pass over the whole batch): 200,000 Galactic
binaries, f0 log-uniform on [1e-4, 2.5e-2] Hz, N chosen per binary by
frequency band from {64, 128, 256, 512, 1024, 2048}, amp log-U(1e-23, 1e-21),
fdot log-U(1e-18, 1e-15), fddot = 11/3 fdot^2/f0, angles isotropic; T = 4 x
31,557,600 s, dt = 5 s; data = the injected sum of all binaries plus
Gaussian noise drawn from the analytic A/E PSD on the full 0-0.1 Hz grid
(L = 12,623,041 bins, A and E, complex128).  Synthetic, seeded.

``value``: binaries/s of the pair-form fused kernel (slow part, FFT and
<d|h> in float-pair arithmetic on the FP32 pipe; one persistent work-queue
launch per step; parameters, data and PSD resident in HBM), the form whose
log-likelihood stays within 1e-6 max(1, <h|h>) of FP64 on this crowded data.
``e2e``: the same metric through ``GBGPU.get_ll`` with the parameters copied
from pinned host memory every step and the log-likelihoods read back.  The
plain-FP64 and the FP32 mixed forms of the same kernel are timed on the same
batch (``fp64_binaries_per_s``, ``mixed_fp32_binaries_per_s``).
``--impl reference`` times the reference's CPU path (its algorithm restated
in the oracle) on the host cores instead, over the whole batch per step.
"""

import argparse
import contextlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

T_OBS = 4 * 31557600.0
DT = 5.0
B_DEFAULT = 200_000
BANDS = [(1e-4, 5e-4, 64), (5e-4, 1e-3, 128), (1e-3, 3e-3, 256), (3e-3, 6e-3, 512),
         (6e-3, 1.2e-2, 1024), (1.2e-2, 2.5e-2 + 1e-12, 2048)]
METRIC = "binaries/s (wave+loglike) & grads/s, mixed vs plain FP64, 1 GB300, <=1e-6 rel ll"


def draw_workload(B, seed):
    rng = np.random.default_rng(seed)
    f0 = 10 ** rng.uniform(-4, np.log10(2.5e-2), B)
    fdot = 10 ** rng.uniform(-18, -15, B)
    p = np.array([10 ** rng.uniform(-23, -21, B), f0, fdot, 11.0 / 3.0 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B))])
    Ns = np.zeros(B, np.int64)
    for lo, hi, n in BANDS:
        Ns[(f0 >= lo) & (f0 < hi)] = n
    assert np.all(Ns > 0)
    return p, Ns


def alg_bytes(Ns):
    """Algorithmic HBM bytes of one fused launch: per binary the A/E data
    (2 x 16 B) and PSD (2 x 8 B) windows of N bins, 9 FP64 parameters and
    two complex128 outputs: 48 N + 72 + 32."""
    return float(np.sum(48 * Ns + 104))


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling while the timed region runs
    (every 20 ms; entering waits for the first sample, and only samples taken
    after that count)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        import torch
        try:
            self.index = "GPU-" + str(torch.cuda.get_device_properties(index).uuid)
        except Exception:
            self.index = str(index)
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
            self.rows = []
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# ------------------------------------------------------------------ CPU side
_SHARED = {}


def _cpu_init(spec):
    """Pool initializer: attach the A/E data and PSD (shared memory written by
    the parent) and load the oracle's C loops, once per worker."""
    from multiprocessing import shared_memory
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fastgb_oracle as O
    O._lib()
    for key, (name, dtype, n) in spec.items():
        # the parent created the segment and unlinks it (the workers share its
        # resource tracker)
        shm = shared_memory.SharedMemory(name=name)
        _SHARED[key] = (shm, np.ndarray((n,), dtype=np.dtype(dtype), buffer=shm.buf))


def _cpu_noop(_):
    return 0


def _cpu_task(args):
    """One chunk of binaries of one N (sorted by f0): the oracle's NumPy
    waveform and its C likelihood loop against the resident data window
    [a, b).  Returns the number of binaries."""
    import fastgb_oracle as O
    p, N, a, b = args
    dA, dE, S = (_SHARED[k][1] for k in ("dA", "dE", "S"))
    O.get_ll(p, [dA[a:b], dE[a:b]], [S[a:b], S[a:b]], N, T=T_OBS, dt=DT, start_freq_ind=a)
    return p.shape[1]


def _cpu_inject_task(args):
    """The A/E windows of one chunk summed into one slice [a, b) of the grid
    (the oracle's waveform and its scatter-add loop)."""
    import fastgb_oracle as O
    p, N = args
    w = O.waveform(p, N, T=T_OBS, dt=DT)
    si = w["start_inds"]
    a, b = int(si.min()), int(si.max()) + N
    tA = np.zeros(b - a, np.complex128)
    tE = np.zeros(b - a, np.complex128)
    B = p.shape[1]
    O.fill_global_native(tA, tE, O.point_major(w["AETf"][:, 0]), O.point_major(w["AETf"][:, 1]),
                         (si - a).astype(np.int32), N, B, np.zeros(B, np.int32), b - a)
    return a, tA, tE


def cpu_tasks(p, Ns, idx, with_window=True):
    """Tasks over the binaries ``idx``: per N (largest first), sorted by f0,
    about 32k samples each (NumPy's (B, 3, N) temporaries stay cache-sized)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fastgb_oracle as O
    L = int(int(T_OBS / DT) / 2) + 1
    tasks = []
    for n in sorted(np.unique(Ns[idx]).tolist(), reverse=True):
        sel = idx[Ns[idx] == n]
        sel = sel[np.argsort(p[1, sel], kind="stable")]
        chunk = max(8, 32768 // n)
        for c in range(0, len(sel), chunk):
            s = sel[c:c + chunk]
            if not with_window:
                tasks.append((p[:, s].copy(), int(n)))
                continue
            si = O.start_indices(p[1, s], n, T_OBS, DT)
            tasks.append((p[:, s].copy(), int(n), max(0, int(si.min()) - 1),
                          min(L, int(si.max()) + n + 1)))
    return tasks


class CpuPool:
    """Spawn pool over the host cores with the A/E data and PSD resident in
    shared memory: each timed pass sends only parameters."""

    def __init__(self, dA, dE, S, workers):
        import multiprocessing as mp
        from multiprocessing import shared_memory
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import fastgb_oracle as O
        O._lib()                              # build the C loops before the workers start
        self.shm, spec = [], {}
        self.arrays = {}
        for key, arr in (("dA", dA), ("dE", dE), ("S", S)):
            shm = shared_memory.SharedMemory(create=True, size=max(1, arr.nbytes))
            view = np.ndarray(arr.shape, arr.dtype, buffer=shm.buf)
            view[:] = arr
            self.shm.append(shm)
            self.arrays[key] = view
            spec[key] = (shm.name, arr.dtype.str, arr.shape[0])
        self.workers = workers
        self.pool = mp.get_context("spawn").Pool(workers, initializer=_cpu_init, initargs=(spec,))
        self.pool.map(_cpu_noop, range(4 * workers), chunksize=1)

    def inject(self, p, Ns):
        """Add the sum of all binaries' A/E windows to the resident data."""
        for a, tA, tE in self.pool.imap_unordered(
                _cpu_inject_task, cpu_tasks(p, Ns, np.arange(p.shape[1]), False)):
            self.arrays["dA"][a:a + len(tA)] += tA
            self.arrays["dE"][a:a + len(tE)] += tE

    def run(self, tasks):
        """One pass over ``tasks``: (wall seconds, binaries)."""
        t0 = time.perf_counter()
        n = sum(self.pool.map(_cpu_task, tasks, chunksize=1))
        return time.perf_counter() - t0, n

    def close(self):
        self.pool.close()
        self.pool.join()
        self.arrays = {}
        for shm in self.shm:
            shm.close()
            shm.unlink()


def cpu_baseline(p, Ns, dA, dE, S, workers, stride=2):
    """The oracle port (the reference's algorithm: NumPy waveform + the C
    likelihood loop) on every ``stride``-th binary of the batch (the same N
    mix) with the data resident in the workers; one warm-up pass, one timed."""
    pool = CpuPool(dA, dE, S, workers)
    try:
        idx = np.arange(0, p.shape[1], stride)
        tasks = cpu_tasks(p, Ns, idx)
        pool.run(tasks[:: max(1, len(tasks) // (4 * workers))])
        wall, n = pool.run(tasks)
    finally:
        pool.close()
    return {"value": n / wall, "unit": "binaries/s", "cores": int(workers), "kind": "port",
            "sample": (f"oracle (NumPy waveform + C get_ll) on every {stride}nd binary of the "
                       f"batch ({n} binaries, the same N mix), {workers} spawn workers with the "
                       f"data in shared memory, wall {wall:.1f} s")}


# ------------------------------------------------------------------ GPU side
def host_noise(seed):
    """Seeded Gaussian A/E noise from the analytic A/E PSD on the 4-yr, 5-s
    grid (rfft bins 0 ... L-1; bin 0 has infinite PSD and no noise), drawn on
    the host so that the GPU arm and the CPU reference arm hold the same
    data.  Returns (A, E, S) NumPy arrays."""
    from gbgpu_gb300.sensitivity import A1TDISens
    T = int(T_OBS / DT) * DT
    L = int(int(T_OBS / DT) / 2) + 1
    f = np.arange(L) / T
    S = np.empty(L)
    S[1:] = A1TDISens.get_Sn(f[1:])
    S[0] = np.inf
    sig = np.sqrt(S * (T / 4.0))
    sig[0] = 0.0
    rng = np.random.default_rng(seed)
    dA = (rng.standard_normal(L) + 1j * rng.standard_normal(L)) * sig
    dE = (rng.standard_normal(L) + 1j * rng.standard_normal(L)) * sig
    return dA, dE, S


def make_noise(seed):
    """host_noise on the device: ([A, E] complex128 tensors, PSD tensor, PSD array)."""
    import torch
    dA, dE, S = host_noise(seed)
    data = [torch.as_tensor(dA, device="cuda"), torch.as_tensor(dE, device="cuda")]
    return data, torch.as_tensor(S, device="cuda"), S


def make_data(gb, p, Ns, seed):
    """Injected sum of all binaries + Gaussian noise from the analytic A/E PSD."""
    import torch
    T = int(T_OBS / DT) * DT
    L = int(int(T_OBS / DT) / 2) + 1
    data, Sd, S = make_noise(seed)
    # the sources, one N class at a time (the FP64 fused fill kernel)
    tmpl = torch.zeros((1, 2, L), dtype=torch.complex128, device="cuda")
    acc = torch.zeros_like(tmpl)
    for n in np.unique(Ns):
        sel = Ns == n
        gb.generate_global_template(p[:, sel].T, np.zeros(int(sel.sum()), np.int32), tmpl,
                                    N=int(n), T=T_OBS, dt=DT, precision="fp64")
        acc += tmpl
    data[0] += acc[0, 0]
    data[1] += acc[0, 1]
    w = 4.0 / T / Sd
    w[0] = 0.0
    d_d = float((w * (data[0].abs() ** 2 + data[1].abs() ** 2)).sum().item())
    return data, Sd, d_d, S


def draw_config0(seed, B=1000):
    """(9, B) parameters of the plain-FP64 workload: amp log-U(1e-23, 1e-21),
    f0 U(1e-3, 5e-3) Hz, fdot log-U(1e-18, 1e-15), fddot = 11/3 fdot^2/f0,
    phi0, lam U[0, 2 pi), psi U[0, pi), iota = arccos U[-1, 1], beta =
    arcsin U[-1, 1]."""
    rng = np.random.default_rng(seed)
    f0 = rng.uniform(1e-3, 5e-3, B)
    fdot = 10 ** rng.uniform(-18, -15, B)
    return np.array([10 ** rng.uniform(-23, -21, B), f0, fdot, 11.0 / 3.0 * fdot ** 2 / f0,
                     rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                     rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                     np.arcsin(rng.uniform(-1, 1, B))])


CFG0_N, CFG0_DT = 128, 10.0


def config0_bench(gb, seed, steps):
    """The plain-FP64 workload: 1,000 binaries, N = 128, dt = 10 s, on the
    4-yr grid from 0 to 0.1 Hz (the same 12,623,041 bins: T is a multiple of
    10 s too; the configuration's 0-0.1 Hz is taken literally although 10 s
    samples put Nyquist at 0.05 Hz); data = the injected sum of the 1,000
    binaries + noise.  A step is run_wave (A/E/T and X/Y/Z windows) and
    get_ll through the class API, parameters on the device.  The CPU leg
    times the oracle's FP64 run_wave + get_ll on one core."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    p = draw_config0(seed)
    B = p.shape[1]
    data, Sd, S = make_noise(seed + 11)
    tmpl = torch.zeros((1, 2, Sd.shape[0]), dtype=torch.complex128, device="cuda")
    gb.generate_global_template(p.T, np.zeros(B, np.int32), tmpl, N=CFG0_N, T=T_OBS, dt=CFG0_DT,
                                precision="fp64")
    data[0] += tmpl[0, 0]
    data[1] += tmpl[0, 1]
    del tmpl
    gb.d_d = 0.0
    prm = torch.as_tensor(p, device="cuda")
    out = {"workload": "1,000 binaries, N=128, T=4x31557600 s, dt=10 s, oversample=1, tdi2=False; "
                       "data = injected sum + noise on the 0-0.1 Hz grid (12,623,041 bins)",
           "steps": steps}

    def step(prec):
        if prec == "fp64":
            gb.run_wave(*prm, N=CFG0_N, T=T_OBS, dt=CFG0_DT)
        gb.get_ll(prm, data, [Sd, Sd], N=CFG0_N, T=T_OBS, dt=CFG0_DT, precision=prec)

    for prec in ("fp64", "pair", "mixed"):
        step(prec)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            step(prec)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        key = "fp64_wave_and_ll" if prec == "fp64" else f"{prec}_ll"
        out[f"{key}_ms"] = ms
        out[f"{key}_binaries_per_s"] = B / (ms / 1e3)
    import fastgb_oracle as O
    dA, dE = data[0].cpu().numpy(), data[1].cpu().numpy()
    O.get_ll(p[:, :50], [dA, dE], [S, S], CFG0_N, T=T_OBS, dt=CFG0_DT)      # warm
    t0 = time.perf_counter()
    O.get_ll(p, [dA, dE], [S, S], CFG0_N, T=T_OBS, dt=CFG0_DT)
    wall = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": B / wall, "unit": "binaries/s", "cores": 1, "kind": "port",
                           "sample": "the whole 1,000-binary batch once: oracle FP64 run_wave "
                                     "(NumPy) + get_ll (C), one core"}
    return out


def sparse_accuracy(gb, p, Ns, Sd, seed, count=2000):
    """max |dlogL| / max(1, <h|h>) of the pair and mixed forms vs FP64 on data
    holding only well-separated sources plus noise: {"pair": x, "mixed": y}."""
    import torch
    Tu = int(T_OBS / DT) * DT
    order = np.argsort(p[1])
    si = np.rint((np.rint(p[1, order] * Tu) - Ns[order] / 2)).astype(np.int64)
    keep, last = [], -10 ** 9
    for j, b in enumerate(order):
        if si[j] > last + 2 * 2048:
            keep.append(b)
            last = si[j] + Ns[b]
        if len(keep) >= count:
            break
    keep = np.array(keep)
    dat, _, _ = make_noise(seed + 7)
    L = Sd.shape[0]
    tmpl = torch.zeros((1, 2, L), dtype=torch.complex128, device="cuda")
    for n in np.unique(Ns[keep]):
        sel = keep[Ns[keep] == n]
        gb.generate_global_template(p[:, sel].T, np.zeros(len(sel), np.int32), tmpl, N=int(n),
                                    T=T_OBS, dt=DT, precision="fp64")
        dat[0] += tmpl[0, 0]
        dat[1] += tmpl[0, 1]
    out = {}
    for prec in ("fp64", "pair", "mixed"):
        gb.get_ll(p[:, keep], dat, [Sd, Sd], N=Ns[keep], T=T_OBS, dt=DT, precision=prec)
        out[prec] = (gb.d_h.real.clone(), gb.h_h.real.clone())
    res = {}
    for prec in ("pair", "mixed"):
        d = (-0.5 * ((out[prec][1] - out["fp64"][1]) - 2 * (out[prec][0] - out["fp64"][0]))).abs()
        res[prec] = (d / torch.clamp(out["fp64"][1], min=1.0)).max().item()
    return res


def time_ll_variants(gb, prm, data, Sd, N, tdi2, steps, tag):
    """Binaries/s of the FP64, pair (9 parameters) and mixed fused likelihood
    and of the likelihood + gradient kernel for the batch ``prm`` (nparams, B)
    at one N, each at its autotuned launch shape (kernel launches through the
    C ABI, inputs on the device).  Returns (rates, launch shapes)."""
    import ctypes
    import torch
    from gbgpu_gb300 import _native as nat
    from gbgpu_gb300.utility import flops_per_binary
    Tu = int(T_OBS / DT) * DT
    NP, B = prm.shape
    L = data[0].shape[0]
    zeros = torch.zeros(B, dtype=torch.int32, device="cuda")
    la = nat.LLArgs()
    la.A_data, la.E_data = data[0].data_ptr(), data[1].data_ptr()
    la.A_psd = la.E_psd = Sd.data_ptr()
    la.data_length, la.num_data, la.num_psd = L, 1, 1
    la.data_index = la.noise_index = zeros.data_ptr()
    la.df = 1.0 / Tu
    d_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    h_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    g = torch.empty((NP, B), dtype=torch.float64, device="cuda")
    lib = nat.lib()
    sh = nat.stream_handle()
    out, shapes = {}, {}
    variants = (("fp64", "fp64"), ("pair", "pair"), ("mixed", "mixed"), ("grad", "mixed"))
    for name, prec in variants:
        if prec == "pair" and NP != 9:
            continue                          # the pair form covers the 9-parameter model
        box = {}

        def set_shape(tile, bps):
            plan = gb._plan(N, Tu, prec, tdi2, NP, tile, bps)
            box["a"] = plan.args(prm, grad=(name == "grad"))

        def run():
            a = box["a"]
            if name == "grad":
                rc = lib.gbx_waveform_ll_grad(ctypes.byref(a), ctypes.byref(la), nat.ptr(d_h),
                                              nat.ptr(h_h), nat.ptr(g), sh)
            else:
                rc = lib.gbx_waveform_ll(ctypes.byref(a), ctypes.byref(la), nat.ptr(d_h),
                                         nat.ptr(h_h), sh)
            nat.check(rc, name)

        shape = (0, 0)
        if gb.autotune:
            from gbgpu_gb300.autotune import default_tuner, workload_key

            def trial(tile, bps):
                set_shape(tile, bps)
                run()
            shape = default_tuner().tune(
                workload_key("grad" if name == "grad" else "ll", N, B, prec, tdi2, NP), trial)
        shapes[name] = {"tile": int(shape[0]), "blocks_per_sm": int(shape[1])}
        set_shape(*shape)
        for _ in range(2):
            run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push(f"{tag}_{name}")
        e0.record()
        for _ in range(steps):
            run()
        e1.record()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[f"{name}_binaries_per_s"] = B / (ms / 1e3)
        if name != "grad":
            out[f"{name}_tflops"] = float(flops_per_binary(N, tdi2, NP == 14, True)) * B / \
                (ms / 1e3) / 1e12
    return out, shapes


def n256_params(seed, B=50_000):
    """(9, B) parameters of the N = 256 batch: f0 uniform on [1e-3, 5e-3] Hz,
    the other parameters as the main batch."""
    rng = np.random.default_rng(seed + 3)
    f0 = rng.uniform(1e-3, 5e-3, B)
    fdot = 10 ** rng.uniform(-18, -15, B)
    return np.array([10 ** rng.uniform(-23, -21, B), f0, fdot, 11.0 / 3.0 * fdot ** 2 / f0,
                     rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                     rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                     np.arcsin(rng.uniform(-1, 1, B))])


def dropin_section(args):
    """The drop-in kernels alone (``--section dropin``): the N = 256 batch's
    point-major templates against seeded noise on the 4-yr grid, no injected
    sources; one JSON line.  A small, quick case for profiling the two entry
    points (about 1 GB on the device)."""
    import torch
    from gbgpu_gb300 import GBGPU
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    data, Sd, _ = make_noise(args.seed)
    out = dropin_kernels(GBGPU(), n256_params(args.seed), data, Sd, max(1, args.steps))
    out["section"] = "dropin"
    return out


def fill_section(args):
    """The template fills alone (``--section fill``): the 50k N = 256 TDI-2
    batch (f0 on [1e-3, 5e-3] Hz) into 64 group templates over the batch's
    band (about 1 GB of templates), group of each binary drawn at random: the
    fused waveform + atomic fill (gbx_waveform_fill, mixed form) and the
    deterministic gather (waveform windows, then fill_det_kernel); one
    untimed call and ``--steps`` timed ones each; one JSON line.  A small
    case for profiling the fill kernels."""
    import torch
    from gbgpu_gb300 import GBGPU
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    p = n256_params(args.seed)
    B, N, G = p.shape[1], 256, 64
    Tu = int(T_OBS / DT) * DT
    q = np.rint(p[1] * Tu).astype(np.int64) - N // 2
    s0 = int(q.min()) - N
    Lb = int(q.max()) + 2 * N - s0
    gb = GBGPU(precision="mixed")
    gi = torch.as_tensor(np.random.default_rng(args.seed + 6).integers(0, G, B), dtype=torch.int32,
                         device="cuda")
    tmpl = torch.zeros((G, 2, Lb), dtype=torch.complex128, device="cuda")
    pT = torch.as_tensor(p.T.copy(), device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    out = {"section": "fill", "binaries": B, "N": N, "groups": G, "band_bins": Lb}

    def timed(run, name):
        run()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(name)
        ev[0].record()
        for _ in range(max(1, args.steps)):
            run()
        ev[1].record()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / max(1, args.steps)

    for mode, sort in (("atomic", False), ("atomic", True), ("deterministic", False)):
        key = mode + ("_sorted" if sort else "")
        out[f"{key}_ms"] = timed(lambda: gb.generate_global_template(
            pT, gi, tmpl, N=N, T=T_OBS, dt=DT, tdi2=True, start_freq_ind=s0, fill_mode=mode,
            sort=sort), f"fill_{key}")
    # dense: the swap sampler's residuals, 512 walkers x 500 sources of N = 512
    # in a 34,000-bin band, added into (A, E) rows of each walker
    W, K, Nd, Ld = 512, 500, 512, 34_000
    rng = np.random.default_rng(args.seed + 8)
    sd = int(2e-3 * Tu)
    f0 = (sd + 1024 + rng.uniform(0, Ld - 2048, W * K)) / Tu
    fdot = 10 ** rng.uniform(-18, -16, W * K)
    pd = torch.as_tensor(np.array([10 ** rng.uniform(-23, -21, W * K), f0, fdot,
                                   11 / 3 * fdot ** 2 / f0, rng.uniform(0, 2 * np.pi, W * K),
                                   np.arccos(rng.uniform(-1, 1, W * K)),
                                   rng.uniform(0, np.pi, W * K), rng.uniform(0, 2 * np.pi, W * K),
                                   np.arcsin(rng.uniform(-1, 1, W * K))]), device="cuda")
    gw = torch.arange(W, device="cuda", dtype=torch.int32).repeat_interleave(K)
    rA = torch.zeros((W, Ld), dtype=torch.complex128, device="cuda")
    rE = torch.zeros_like(rA)
    out["dense"] = {"workload": f"{W} groups x {K} sources, N={Nd}, {Ld}-bin band, mixed form"}
    for sort in (False, True):
        out["dense"]["sorted_ms" if sort else "unsorted_ms"] = timed(
            lambda: gb.add_to_templates(pd, gw, (rA, rE), N=Nd, T=T_OBS, dt=DT, start_freq_ind=sd,
                                        sort=sort), "dense_sorted" if sort else "dense_unsorted")
    return out


def pair_section(args):
    """The headline kernel alone (``--section pair``): the uneven-N workload's
    first ``--binaries`` binaries (20,000 gives a small case of about 1 GB on
    the device) against seeded noise on the 4-yr grid, through
    gbx_waveform_ll in the pair form at the bench's launch shape (tile 2048),
    one untimed call and ``--steps`` timed ones; one JSON line."""
    import ctypes
    import torch
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300 import _native as nat
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    p, Ns = draw_workload(args.binaries, args.seed)
    data, Sd, _ = make_noise(args.seed)
    Tu = int(T_OBS / DT) * DT
    gb = GBGPU()
    B = p.shape[1]
    prm = torch.as_tensor(p, device="cuda").contiguous()
    zeros = torch.zeros(B, dtype=torch.int32, device="cuda")
    la = gb._ll_args(data, [Sd, Sd], data[0].shape[0], zeros, zeros, Tu)
    a = gb._plan(Ns, Tu, "pair", False, 9, 2048, 0).args(prm)
    d_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    h_h = torch.empty(B, dtype=torch.complex128, device="cuda")

    def run():
        nat.check(nat.lib().gbx_waveform_ll(ctypes.byref(a), ctypes.byref(la), nat.ptr(d_h),
                                            nat.ptr(h_h), nat.stream_handle()), "gbx_waveform_ll")
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(max(1, args.steps)):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(1, args.steps)
    return {"section": "pair", "binaries": B, "samples": int(Ns.sum()), "ms": ms,
            "binaries_per_s": B / (ms / 1e3), "alg_bytes": alg_bytes(Ns)}


def n256_tdi2_bench(gb, data, Sd, seed, steps):
    """50,000 binaries, N = 256, TDI-2, f0 uniform on [1e-3, 5e-3] Hz and the
    other parameters as the main batch, on the same 4-yr data grid.  Times the FP64 and
    mixed fused likelihood and the likelihood + gradient kernel."""
    import torch
    p = n256_params(seed)
    prm = torch.as_tensor(p, device="cuda").contiguous()
    Tu = int(T_OBS / DT) * DT
    out = {"workload": "50,000 binaries, N=256, tdi2=True, T=4x31557600 s",
           "steps": steps}
    rates, shapes = time_ll_variants(gb, prm, data, Sd, 256, True, steps, "n256")
    out.update(rates)
    out["launch_shapes"] = shapes
    out["grad_over_forward"] = out["grad_binaries_per_s"] / out["mixed_binaries_per_s"]
    out["mixed_over_fp64"] = out["mixed_binaries_per_s"] / out["fp64_binaries_per_s"]
    out["pair_over_fp64"] = out["pair_binaries_per_s"] / out["fp64_binaries_per_s"]
    out["dropin"] = dropin_kernels(gb, p, data, Sd, steps)
    out["fisher"] = fisher_bench(gb, p, Tu)
    out["hmc"] = hmc_bench(gb, p, data, Sd, seed)
    out["ensemble"] = ensemble_bench(gb, p, data, Sd, seed)
    return out


def thirdbody_n256_bench(data, Sd, seed, steps):
    """GBGPUThirdBody: 50,000 binaries with a third body, N = 256, TDI-2, the
    binary parameters as the N = 256 batch, A2 log-uniform on [1, 1e4] m/s,
    varpi uniform, e2 uniform on [0, 0.9], P2 log-uniform on [1, 40] yr, T2
    uniform on [0, P2], on the same 4-yr data grid.  Times the FP64 and mixed fused likelihood and the
    likelihood + gradient kernel (14 parameters)."""
    import torch
    from gbgpu_gb300 import GBGPUThirdBody
    rng = np.random.default_rng(seed + 5)
    B = 50_000
    f0 = rng.uniform(1e-3, 5e-3, B)
    fdot = 10 ** rng.uniform(-18, -15, B)
    P2 = 10 ** rng.uniform(0, np.log10(40), B)
    p = np.array([10 ** rng.uniform(-23, -21, B), f0, fdot, 11.0 / 3.0 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B)), 10 ** rng.uniform(0, 4, B),
                  rng.uniform(0, 2 * np.pi, B), rng.uniform(0, 0.9, B), P2,
                  rng.uniform(0, 1, B) * P2])
    gb = GBGPUThirdBody(precision="mixed", autotune=True)
    prm = torch.as_tensor(p, device="cuda").contiguous()
    out = {"workload": "GBGPUThirdBody, 50,000 binaries, N=256, tdi2=True, T=4x31557600 s",
           "steps": steps}
    rates, shapes = time_ll_variants(gb, prm, data, Sd, 256, True, steps, "thirdbody_n256")
    out.update(rates)
    out["launch_shapes"] = shapes
    out["grad_over_forward"] = out["grad_binaries_per_s"] / out["mixed_binaries_per_s"]
    out["mixed_over_fp64"] = out["mixed_binaries_per_s"] / out["fp64_binaries_per_s"]
    return out


FREE8 = (0, 1, 2, 4, 5, 6, 7, 8)      # amp, f0, fdot, phi0, iota, psi, lam, beta (fddot fixed)


def dropin_kernels(gb, p, data, Sd, steps):
    """The reference's two native entry points as replaced here (gbx_get_ll,
    gbx_fill_global through the backend method table) on the 50k N = 256 batch:
    point-major FP64 templates from run_wave, then the unfused likelihood and
    the scatter-add into 256 template groups.  Algorithmic bytes per binary:
    get_ll 80 N + 44 (template, data, PSD windows, indices, outputs),
    fill_global 96 N (template read + read-modify-write of the globals)."""
    import torch
    from gbgpu_gb300.backend import get_backend
    be = get_backend()
    B, N = p.shape[1], 256
    gb.run_wave(*p, N=N, T=T_OBS, dt=DT, tdi2=True)
    A_pm, E_pm = gb.A_out.contiguous(), gb.E_out.contiguous()    # point-major, i*B + b
    start = gb.start_inds.to(torch.int32).contiguous()
    L = data[0].shape[0]
    zeros = torch.zeros(B, dtype=torch.int32, device="cuda")
    d_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    h_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    Tu = int(T_OBS / DT) * DT
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timeit(fn, name):
        fn()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(name)
        ev[0].record()
        for _ in range(steps):
            fn()
        ev[1].record()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / steps

    ms_ll = timeit(lambda: be.get_ll(d_h, h_h, A_pm, E_pm, data[0], data[1], Sd, Sd, 1.0 / Tu,
                                     start, N, B, zeros, zeros, L), "dropin_get_ll")
    ms_ll64 = timeit(lambda: be.get_ll(d_h, h_h, A_pm, E_pm, data[0], data[1], Sd, Sd, 1.0 / Tu,
                                       start, N, B, zeros, zeros, L, fp64=True),
                     "dropin_get_ll_fp64")
    G = 256
    Lf = int(start.max().item()) + N + 1
    glob = torch.zeros((2, G * Lf), dtype=torch.complex128, device="cuda")
    gi = torch.as_tensor(np.random.default_rng(5).integers(0, G, B), dtype=torch.int32,
                         device="cuda")
    ms_fill = timeit(lambda: be.fill_global(glob[0], glob[1], A_pm, E_pm, start, N, B, gi, Lf),
                     "dropin_fill_global")
    peak, src = hbm_peak()
    ll_bytes = B * (80.0 * N + 44)
    fill_bytes = B * 96.0 * N
    return {"workload": f"{B} binaries, N={N}, point-major FP64 templates",
            "get_ll_ms": ms_ll, "get_ll_GBps": ll_bytes / (ms_ll / 1e3) / 1e9,
            "get_ll_frac": ll_bytes / (ms_ll / 1e3) / 1e9 / peak,
            "get_ll_fp64_ms": ms_ll64,
            "fill_global_ms": ms_fill, "fill_global_GBps": fill_bytes / (ms_fill / 1e3) / 1e9,
            "fill_global_frac": fill_bytes / (ms_fill / 1e3) / 1e9 / peak,
            "peak_GBps": peak, "note": f"peak {src}; algorithmic bytes (80 N + 44 and 96 N per "
                                       "binary) over CUDA-event time"}


def fisher_bench(gb, p, Tu):
    """Per-binary 8x8 Fisher matrices of the 50k N = 256 binaries (TDI-2):
    in-kernel forward mode (one gbx_fisher launch) and, for comparison, FP64
    five-point differences of the batched waveform."""
    import torch
    B = p.shape[1]
    out = {"binaries": B, "params": len(FREE8)}
    Fs = {}
    for method in ("forward", "differences"):
        # untimed call on a slice: one-time costs (library kernels loaded on first
        # use, plans, orbit tables) stay out of the timing
        gb.fisher_matrices(p[:, :512], N=256, T=T_OBS, dt=DT, tdi2=True, inds=FREE8,
                           return_gpu=True, method=method)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push(f"n256_fisher_{method}")
        Fs[method] = gb.fisher_matrices(p, N=256, T=T_OBS, dt=DT, tdi2=True, inds=FREE8,
                                        return_gpu=True, method=method)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        dt_s = time.perf_counter() - t0
        out[f"{method}_seconds"] = dt_s
        out[f"{method}_binaries_per_s"] = B / dt_s
    d = torch.sqrt(torch.diagonal(Fs["differences"], dim1=1, dim2=2))
    diff = (Fs["forward"] - Fs["differences"]).abs() / (d[:, :, None] * d[:, None, :])
    out.update({"seconds": out["forward_seconds"], "binaries_per_s": out["forward_binaries_per_s"],
                "finite": bool(torch.isfinite(Fs["forward"]).all().item()),
                "max_forward_vs_differences": float(diff.max().item()),
                "note": "forward: one gbx_fisher launch (14 transforms per binary, 45 products "
                        "per channel and bin) plus prep; differences: 32 batched FP64 waveform launches + one "
                        "einsum; host wall time after one untimed call on 512 binaries; "
                        "difference normalised by sqrt(F_ii F_jj)"})
    return out


def hmc_bench(gb, p, data, Sd, seed, B=4096, transitions=100, n_leapfrog=10, step=0.2):
    """1,000-step HMC leapfrog chains for 4,096 binaries in one CUDA graph: the
    4,096 loudest of the 50k N = 256 binaries, injected into a copy of the data; mass
    metric from their Fisher diagonals; every leapfrog step is one fused
    likelihood + gradient launch."""
    import torch
    from gbgpu_gb300.mcmc import HMCSampler
    sel = np.argsort(-p[0])[:B]
    q = np.ascontiguousarray(p[:, sel])
    dA, dE = data[0].clone(), data[1].clone()
    gb.add_to_templates(torch.as_tensor(q, device="cuda"), torch.zeros(B, dtype=torch.int32,
                                                                    device="cuda"),
                        (dA[None], dE[None]), N=256, T=T_OBS, dt=DT, tdi2=True, precision="fp64")
    F = gb.fisher_matrices(q, N=256, T=T_OBS, dt=DT, tdi2=True, inds=FREE8, return_gpu=True)
    sig = 1.0 / torch.sqrt(torch.diagonal(F, dim1=1, dim2=2)).T.contiguous()
    d_d = gb.d_d
    gb.d_d = 0.0
    smp = HMCSampler(gb, torch.as_tensor(q, device="cuda"), [dA, dE], [Sd, Sd], N=256, T=T_OBS,
                     dt=DT, scales=sig, step_size=step, n_leapfrog=n_leapfrog, tdi2=True,
                     free=FREE8)
    gb.d_d = d_d
    g = torch.Generator(device="cuda")
    g.manual_seed(seed + 33)
    moms = torch.randn((transitions, len(FREE8), B), generator=g, device="cuda",
                       dtype=torch.float64)
    lus = torch.log(torch.rand((transitions, B), generator=g, device="cuda",
                               dtype=torch.float64).clamp_min(1e-300))
    smp.capture(moms, lus)
    smp.accepted.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("n256_hmc")
    e0.record()
    smp.replay()
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    steps = transitions * n_leapfrog
    return {"binaries": B, "leapfrog_steps": steps, "transitions": transitions,
            "step_size": step, "graph_ms": ms,
            "binary_leapfrog_steps_per_s": B * steps / (ms / 1e3),
            "acceptance": float(smp.accepted.sum().item()) / (B * transitions),
            "note": "whitened coordinates (Fisher-diagonal sigmas); one fused likelihood + "
                    "gradient launch per leapfrog step, all captured in one CUDA graph"}


def ensemble_bench(gb, p, data, Sd, seed, B=512, W=64, steps=50):
    """Stretch-move ensembles (affine-invariant, Goodman & Weare): the 512
    loudest of the 50k N = 256 binaries, injected into a copy of the data, 64
    walkers each started in a 0.1-sigma ball of their Fisher diagonals; 50
    steps (100 fused likelihood launches of 16,384 points) in one CUDA graph."""
    import torch
    from gbgpu_gb300.mcmc import StretchSampler, stretch_draws
    sel = np.argsort(-p[0])[:B]
    q = np.ascontiguousarray(p[:, sel])
    dA, dE = data[0].clone(), data[1].clone()
    gb.add_to_templates(torch.as_tensor(q, device="cuda"),
                        torch.zeros(B, dtype=torch.int32, device="cuda"),
                        (dA[None], dE[None]), N=256, T=T_OBS, dt=DT, tdi2=True, precision="fp64")
    F = gb.fisher_matrices(q, N=256, T=T_OBS, dt=DT, tdi2=True, inds=FREE8, return_gpu=True)
    sig = (1.0 / torch.sqrt(torch.diagonal(F, dim1=1, dim2=2))).T
    g = torch.Generator(device="cuda")
    g.manual_seed(seed + 55)
    x = torch.as_tensor(q, device="cuda")[:, :, None].repeat(1, 1, W)
    x[list(FREE8)] += 0.1 * sig[:, :, None] * torch.randn((len(FREE8), B, W), generator=g,
                                                          device="cuda", dtype=torch.float64)
    d_d = gb.d_d
    gb.d_d = 0.0
    smp = StretchSampler(gb, x, [dA, dE], [Sd, Sd], N=256, T=T_OBS, dt=DT, tdi2=True, free=FREE8)
    gb.d_d = d_d
    u, j, lu = stretch_draws(steps, B, W // 2, g, "cuda")
    smp.capture(u, j, lu)
    smp.accepted.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("n256_ensemble")
    e0.record()
    smp.replay()
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"binaries": B, "walkers": W, "steps": steps, "graph_ms": ms,
            "walker_steps_per_s": B * W * steps / (ms / 1e3),
            "acceptance": float(smp.accepted.sum().item()) / (B * W * steps),
            "note": "stretch move, two half-ensemble updates per step, each one fused "
                    "likelihood launch over all binaries; all steps captured in one CUDA graph"}


def fill_bench(gb, seed, B=1_000_000, G=256, N=256, steps=3):
    """Global templates of 1e6 binaries: f0 density f^(-11/3) on [1e-4, 1e-2] Hz,
    amp ~ f0^(2/3) with log-normal scatter (sigma 0.3), N = 256, group index
    uniform over 256 walkers, templates (256, 2, 12,623,041) complex128
    (103.4 GB).  Times the fused atomic fill and the deterministic fill
    (waveforms, sort by (group, start), ordered gather); the zeroing of the
    templates that the atomic mode needs is timed separately."""
    import torch
    rng = np.random.default_rng(seed + 2)
    lo, hi = 1e-4, 1e-2
    u = rng.uniform(0, 1, B)
    f0 = (lo ** (-8 / 3) - u * (lo ** (-8 / 3) - hi ** (-8 / 3))) ** (-3 / 8)
    fdot = 10 ** rng.uniform(-18, -15, B)
    amp = 1e-22 * (f0 / 1e-3) ** (2 / 3) * np.exp(0.3 * rng.standard_normal(B))
    p = np.array([amp, f0, fdot, 11.0 / 3.0 * fdot ** 2 / f0, rng.uniform(0, 2 * np.pi, B),
                  np.arccos(rng.uniform(-1, 1, B)), rng.uniform(0, np.pi, B),
                  rng.uniform(0, 2 * np.pi, B), np.arcsin(rng.uniform(-1, 1, B))])
    gi = torch.as_tensor(rng.integers(0, G, B).astype(np.int32), device="cuda")
    pT = torch.as_tensor(p.T.copy(), device="cuda")
    L = int(int(T_OBS / DT) / 2) + 1
    out = {"workload": f"{B} binaries (f^-11/3 on 1e-4..1e-2 Hz), N={N}, {G} groups x 2 x {L} "
                       "complex128 templates", "steps": steps}
    try:
        tmpl = torch.empty((G, 2, L), dtype=torch.complex128, device="cuda")
    except RuntimeError as e:
        out["unavailable"] = f"template allocation failed: {e}"[:200]
        return out
    out["template_GB"] = tmpl.numel() * 16 / 1e9
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timeit(fn, name):
        fn()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(name)
        ev[0].record()
        for _ in range(steps):
            fn()
        ev[1].record()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / steps

    ms_zero = timeit(lambda: tmpl.zero_(), "fill_zero")
    for prec in ("fp64", "pair", "mixed"):
        for mode in ("atomic", "deterministic"):
            ms = timeit(lambda: gb.generate_global_template(pT, gi, tmpl, N=N, T=T_OBS, dt=DT,
                                                            precision=prec, fill_mode=mode),
                        f"fill_{prec}_{mode}")
            out[f"{prec}_{mode}_ms"] = ms
            out[f"{prec}_{mode}_binaries_per_s"] = B / (ms / 1e3)
    out["zeroing_ms"] = ms_zero
    out["note"] = ("templates accumulate in FP64 in every variant; fp64/pair/mixed is the "
                   "waveform precision.  atomic includes zeroing channels 0/1 (the reference's "
                   "overwrite semantics); deterministic writes every bin itself")
    del tmpl
    torch.cuda.empty_cache()
    return out


def swap_bench(seed, W=4096, K=500, N=512, steps=100, replays=3):
    """GBGPUThirdBody swap sampler: 4,096 walkers x 500 sources, N = 512,
    T = 4 yr, dt = 5 s; every walker proposes a swap of one source per step
    (swap likelihood in the mixed form, Metropolis accept, residual update);
    100 steps are captured as one CUDA graph and replayed.  Sources sit in a
    ~2.5e-4 Hz band (34,000 bins) of seeded noise.  Reports swaps/s."""
    import torch
    from gbgpu_gb300 import GBGPUThirdBody
    from gbgpu_gb300.mcmc import SwapSampler, random_proposals, log_uniforms
    from gbgpu_gb300.sensitivity import A1TDISens
    rng = np.random.default_rng(seed + 4)
    Tu = int(T_OBS / DT) * DT
    s0 = int(2e-3 * Tu)
    Lb = 34_000
    f0 = (s0 + 1024 + rng.uniform(0, Lb - 2048, (W, K))) / Tu
    fdot = 10 ** rng.uniform(-18, -16, (W, K))
    P2 = 10 ** rng.uniform(0, np.log10(40), (W, K))
    p = np.stack([10 ** rng.uniform(-23, -21, (W, K)), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, (W, K)), np.arccos(rng.uniform(-1, 1, (W, K))),
                  rng.uniform(0, np.pi, (W, K)), rng.uniform(0, 2 * np.pi, (W, K)),
                  np.arcsin(rng.uniform(-1, 1, (W, K))), 10 ** rng.uniform(-2, 2, (W, K)),
                  rng.uniform(0, 2 * np.pi, (W, K)), rng.uniform(0, 0.9, (W, K)), P2,
                  rng.uniform(0, 1, (W, K)) * P2])
    S = A1TDISens.get_Sn((np.arange(Lb) + s0) / Tu)
    Sd = torch.as_tensor(S, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(seed + 44)
    sig = torch.sqrt(Sd * (Tu / 4.0))
    data = [torch.complex(torch.randn(Lb, generator=g, device="cuda", dtype=torch.float64) * sig,
                          torch.randn(Lb, generator=g, device="cuda", dtype=torch.float64) * sig)
            for _ in range(2)]
    gb = GBGPUThirdBody(precision="mixed")
    smp = SwapSampler(gb, torch.as_tensor(p, device="cuda"), data, [Sd, Sd], N=N, T=T_OBS,
                      dt=DT, start_freq_ind=s0)
    scale = torch.tensor([0.05, 2e-9, 0, 0, 0.2, 0.1, 0.1, 0.02, 0.02, 0.05, 0.1, 0.02, 0.01, 0.01],
                         dtype=torch.float64, device="cuda")
    ks = [int(x) for x in rng.integers(0, K, steps)]
    props = torch.stack([random_proposals(smp.params[:, :, k], scale, g) for k in ks])
    props[:, 11].clamp_(0.0, 0.9)
    lus = log_uniforms(W, steps, g, "cuda")
    smp.capture(ks, props, lus)
    smp.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("swap_graph")
    e0.record()
    for _ in range(replays):
        smp.replay()
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / replays
    # swap likelihood with its gradient in the proposal (both launches of
    # gbx_swap_ll_grad) for every walker's first proposal, on the current state
    k0 = ks[0]
    old = smp.params[:, :, k0].contiguous()
    prop = props[0].contiguous()
    kw = dict(data_index=smp.walkers, start_freq_ind=s0, N=N, T=T_OBS, dt=DT, return_tensor=True)
    for _ in range(3):
        gb.swap_likelihood(old, prop, [smp.res[0], smp.res[1]], [Sd, Sd], grad=True, **kw)
    torch.cuda.synchronize()
    reps = 20
    e0.record()
    for _ in range(reps):
        gb.swap_likelihood(old, prop, [smp.res[0], smp.res[1]], [Sd, Sd], grad=True, **kw)
    e1.record()
    torch.cuda.synchronize()
    gms = e0.elapsed_time(e1) / reps
    return {"workload": f"GBGPUThirdBody, {W} walkers x {K} sources, N={N}, dt=5 s; "
                        f"{steps} swap steps per CUDA graph", "graph_ms": ms,
            "swaps_per_s": W * steps / (ms / 1e3),
            "acceptance": float(smp.accepted.sum().item()) / (W * steps * (replays + 1)),
            "swap_grad_ms": gms,
            "swaps_with_grad_per_s": W / (gms / 1e3),
            "swap_grad_note": f"{W} (old, new) pairs per call: dlogL and its 14-parameter "
                              "gradient in the proposal (mixed form, eager calls)"}


HEADLINE = "pair"      # the precision whose logL meets <= 1e-6 max(1, <h|h>) on this data


def accuracy(dh, hh, dh64, hh64, ddw=None):
    """max |dlogL| / max(1, <h|h>) against the FP64 form (and / max(1, <h|h>,
    <d|d>_window) when ddw is given)."""
    import torch
    dl = (-0.5 * (hh.real - hh64.real) + (dh.real - dh64.real)).abs()
    out = {"max_dlogL_over_max1_hh": (dl / torch.clamp(hh64.real, min=1.0)).max().item(),
           "count_over_1e-6": int((dl / torch.clamp(hh64.real, min=1.0) > 1e-6).sum().item())}
    if ddw is not None:
        out["max_dlogL_over_max1_hh_ddwindow"] = \
            (dl / torch.clamp(torch.maximum(hh64.real, ddw), min=1.0)).max().item()
    return out


def run_gpu(args, rank, world):
    import torch
    from gbgpu_gb300 import GBGPU, sharding
    from gbgpu_gb300 import _native as nat
    import ctypes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    B = args.binaries
    p, Ns = draw_workload(B, args.seed + rank)
    gb = GBGPU(precision=HEADLINE, autotune=not args.no_autotune)
    data, Sd, d_d, S_host = make_data(gb, p, Ns, args.seed + rank)
    gb.d_d = d_d
    L = data[0].shape[0]

    params_d = torch.as_tensor(p, device="cuda").contiguous()
    Tu_ = int(T_OBS / DT) * DT
    d_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    h_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    zeros = torch.zeros(B, dtype=torch.int32, device="cuda")
    la = nat.LLArgs()
    la.A_data, la.E_data = data[0].data_ptr(), data[1].data_ptr()
    la.A_psd = la.E_psd = Sd.data_ptr()
    la.data_length, la.num_data, la.num_psd = L, 1, 1
    la.data_index = la.noise_index = zeros.data_ptr()
    la.df = 1.0 / (int(T_OBS / DT) * DT)
    lib = nat.lib()
    stream = torch.cuda.current_stream()
    sh = nat.stream_handle(stream)
    grad_out = torch.empty((9, B), dtype=torch.float64, device="cuda")
    variants = ("pair", "mixed", "fp64", "grad")

    def set_shape(prec, tile, bps):
        plan = gb._plan(Ns, Tu_, "mixed" if prec == "grad" else prec, False, 9, tile, bps)
        wargs[prec] = plan.args(params_d, grad=(prec == "grad"))

    wargs = {}
    for prec in variants:
        set_shape(prec, 0, 0)

    def step(prec):
        if prec == "grad":
            rc = lib.gbx_waveform_ll_grad(ctypes.byref(wargs["grad"]), ctypes.byref(la),
                                          ctypes.c_void_p(d_h.data_ptr()),
                                          ctypes.c_void_p(h_h.data_ptr()),
                                          ctypes.c_void_p(grad_out.data_ptr()), sh)
        else:
            rc = lib.gbx_waveform_ll(ctypes.byref(wargs[prec]), ctypes.byref(la),
                                     ctypes.c_void_p(d_h.data_ptr()), ctypes.c_void_p(h_h.data_ptr()), sh)
        if rc:
            nat.check(rc, "gbx_waveform_ll")

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(prec, K, W, clk=None):
        for _ in range(W):
            step(prec)
        torch.cuda.synchronize()
        sharding.barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(K)]
        with (clk if clk is not None else contextlib.nullcontext()):
            t_wall = time.perf_counter()
            torch.cuda.nvtx.range_push(f"ll_{prec}")   # ncu --nvtx-include ll_<prec>/
            for a, b in ev:
                flush.zero_()                     # evict L2 between timed steps
                a.record(stream)
                step(prec)
                b.record(stream)
            torch.cuda.nvtx.range_pop()
            torch.cuda.synchronize()
            t_wall = time.perf_counter() - t_wall
        ms = [a.elapsed_time(b) for a, b in ev]
        return float(np.mean(ms)), t_wall

    # launch shapes: picked by the autotuner on this batch (same keys as the
    # class API, so the e2e calls below reuse them), else the defaults
    shapes = {}
    if not args.no_autotune:
        from gbgpu_gb300.autotune import default_tuner, workload_key

        for prec in variants:
            kind = "grad" if prec == "grad" else "ll"
            pr = "mixed" if prec == "grad" else prec

            def run(tile, bps, prec=prec):
                set_shape(prec, tile, bps)
                step(prec)
            shapes[prec] = default_tuner().tune(workload_key(kind, Ns, B, pr, False, 9), run)
            set_shape(prec, *shapes[prec])
    torch.cuda.synchronize()

    # accuracy of the pair and mixed forms on the full batch against the FP64 form
    res = {}
    for prec in ("fp64", "pair", "mixed"):
        step(prec)
        torch.cuda.synchronize()
        res[prec] = (d_h.clone(), h_h.clone())
    # <d|d> restricted to each template window (the data's own SNR^2 there)
    Tu = int(T_OBS / DT) * DT
    w = 4.0 / Tu / Sd
    w[0] = 0.0
    cs = torch.cumsum(w * (data[0].abs() ** 2 + data[1].abs() ** 2), 0)
    cs = torch.cat([torch.zeros(1, device="cuda", dtype=cs.dtype), cs])
    si = torch.as_tensor(np.rint(np.rint(p[1] * Tu) - Ns / 2).astype(np.int64), device="cuda")
    nn = torch.as_tensor(Ns, device="cuda")
    ddw = cs[torch.clamp(si + nn, 0, L)] - cs[torch.clamp(si, 0, L)]
    acc = {prec: accuracy(*res[prec], *res["fp64"], ddw) for prec in ("pair", "mixed")}
    sparse = sparse_accuracy(gb, p, Ns, Sd, args.seed + rank)
    for prec in ("pair", "mixed"):
        acc[prec]["sparse_max_dlogL_over_max1_hh"] = sparse[prec]
    del res

    clk = ClockSampler(torch.cuda.current_device())
    ms_head, wall_head = timed(HEADLINE, args.steps, args.warmup, clk)
    ms_mixed, _ = timed("mixed", max(1, min(args.steps, 20)), 1)
    ms_fp64, _ = timed("fp64", max(1, min(args.steps, 3)), 1)
    ms_grad, _ = timed("grad", max(1, min(args.steps, 10)), 1)
    cfg0 = config0_bench(GBGPU(), args.seed + rank, max(1, min(args.steps, 10)))
    cfg3 = n256_tdi2_bench(gb, data, Sd, args.seed + rank, max(1, min(args.steps, 10)))
    cfg3tb = thirdbody_n256_bench(data, Sd, args.seed + rank, max(1, min(args.steps, 10)))
    cfg2 = cfg4 = None
    if not args.no_fill_bench:
        cfg2 = fill_bench(gb, args.seed + rank)
    if not args.no_mcmc_bench:
        cfg4 = swap_bench(args.seed + rank)

    # e2e through the public API: host params -> device, like -> host
    p_pin = torch.from_numpy(np.ascontiguousarray(p)).pin_memory()
    for _ in range(max(1, args.warmup)):
        gb.get_ll(p_pin, data, [Sd, Sd], N=Ns, T=T_OBS, dt=DT, precision=HEADLINE)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gb.get_ll(p_pin, data, [Sd, Sd], N=Ns, T=T_OBS, dt=DT, precision=HEADLINE)
    e2e_s = (time.perf_counter() - t0) / args.steps

    # weak scaling: every rank times its own batch; the job's step time is the
    # slowest rank's
    t_max, e2e_max = sharding.max_over_ranks([ms_head, e2e_s], device="cuda")
    value = world * B / (t_max / 1e3)
    ab = alg_bytes(Ns)
    achieved = ab / (ms_head / 1e3) / 1e9
    peak, peak_src = hbm_peak()
    traffic = profiled("dram_bytes_per_launch")
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "binaries/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_max,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 pairs (slow part, FFT and <d|h> in float-pair arithmetic on the FP32 "
                 "pipe, ~44 bits); FP64 start indices, scalings and outputs",
        "data": "synthetic (seeded binaries; injected sum + Gaussian noise from the analytic A/E PSD)",
        "config": workload_config(B, Ns),
        "precision": HEADLINE,
        "parallelism": f"replicas x{world} (binaries sharded, no collective)",
        "gpu_launches": 2 * args.steps,
        "gpu_launches_note": "per step: prep_kernel (per-binary constants) + pair_kernel<LL>",
        "fp64_binaries_per_s": B / (ms_fp64 / 1e3),
        "pair_over_fp64": ms_fp64 / ms_head,
        "mixed_fp32_binaries_per_s": B / (ms_mixed / 1e3),
        "accuracy": {
            "pair": acc["pair"], "mixed_fp32": acc["mixed"],
            "note": "vs the FP64 form of the same kernels (itself within 1e-10 of the "
                    "reference) on this step's data (the injected sum of all binaries + "
                    "noise); sparse = 2000 non-overlapping sources + noise.  The pair form "
                    "meets |dlogL| <= 1e-6 max(1, <h|h>); the FP32 mixed form's stated bound "
                    "is |dlogL| <= 1e-6 max(1, <h|h>, <d|d>_window)"},
        "grads_per_s": B / (ms_grad / 1e3),
        "grads_note": "binaries/s of the fused likelihood + 9-parameter gradient kernel "
                      "(FP32 mixed form) on the same batch",
        "launch_shapes": {k: {"tile": int(v[0]), "blocks_per_sm": int(v[1])}
                          for k, v in shapes.items()} or "defaults (tile 512, full occupancy)",
        "plain_fp64_1000": cfg0,
        "n256_tdi2": cfg3,
        "fill_templates": cfg2,
        "thirdbody_swaps": cfg4,
        "thirdbody_n256": cfg3tb,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "issue_active_frac": profiled("issue_active_frac"),
                     "note": f"peak {peak_src}; achieved = algorithmic bytes (48 N + 104 per "
                             "binary) / the timed step (prep_kernel + pair_kernel); traffic = "
                             "ncu DRAM bytes per launch (profiles/pair_ll_200k.txt).  The kernel "
                             "is instruction-issue bound on the FP32/ALU pipes (float-pair "
                             "arithmetic; issue_active_frac from ncu), so the HBM fraction is "
                             "low by construction"},
        "compute": compute_roofline(Ns, t_max, clk),
        "issue": issue_roofline(Ns, ms_head, clk),
        "e2e": {"value": world * B / e2e_max, "unit": "binaries/s",
                "h2d_bytes_per_step": int(p.nbytes), "d2h_bytes_per_step": int(B * 8)},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(p, Ns, data[0].cpu().numpy(), data[1].cpu().numpy(),
                                           S_host, workers=args.cpu_workers)
    return out


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback (6.8 TB/s)"


def compute_roofline(Ns, ms, clk):
    """The step's algorithmic FLOPs (``flops_per_binary``: waveform + likelihood,
    the restated formula, not the instructions the kernel issues) over its
    time, against the nominal FP32 rate of the device (SMs x 128 lanes x 2 x
    the maximum SM clock sampled)."""
    import torch
    from gbgpu_gb300.utility import flops_per_binary
    F = float(np.sum(flops_per_binary(Ns, likelihood=True)))
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    mhz = (clk.summary() or {}).get("sm_max_mhz") or 2070.0
    peak = props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12
    achieved = F / (ms / 1e3) / 1e12
    return {"flops_per_step": F, "achieved": achieved, "unit": "TFLOP/s", "peak": peak,
            "frac": achieved / peak,
            "note": "algorithmic FLOPs (gbgpu_gb300.utility.flops_per_binary) per timed step; "
                    "peak = nominal FP32 (SMs x 128 x 2 x max SM clock), not measured"}


def issue_roofline(Ns, ms, clk, sms=None):
    """The bound of the issue-limited pair kernel: its warp instructions per
    step (``warp_instr_per_sample`` of the committed ncu summary, counted on a
    20k-binary slice of the same workload, times the step's samples) over the
    timed step, against the SMs' issue ceiling of one warp instruction per
    cycle on each of an SM's four schedulers at the median SM clock sampled
    during the timed steps."""
    per = profiled("warp_instr_per_sample")
    if per is None:
        return None
    if sms is None:
        import torch
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    summ = clk.summary() or {}
    mhz = summ.get("sm_mhz") or summ.get("sm_max_mhz") or 2070.0
    peak = sms * 4 * mhz * 1e6
    achieved = per * float(np.sum(Ns)) / (ms / 1e3)
    return {"warp_instr_per_sample": per, "achieved": achieved, "unit": "warp instructions/s",
            "peak": peak, "frac": achieved / peak,
            "note": "peak = SMs x 4 schedulers x 1 warp instruction per cycle x median SM clock "
                    "under load; the pair kernel's FP32 float-pair arithmetic is bound here, "
                    "not by HBM"}


def profiled(key, name="pair_ll_200k.txt"):
    """A figure of the committed ncu summary of the headline kernel (a line
    ``key: value``): ``dram_bytes_per_launch`` (dram__bytes_read.sum +
    dram__bytes_write.sum per full-size launch), ``issue_active_frac`` or
    ``warp_instr_per_sample``."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def workload_config(B, Ns):
    """The ``config`` of both arms' JSON lines (the workload, not the arm)."""
    return {"workload": f"{B} binaries, uneven N in {{64..2048}} by f0 band, T=4x31557600 s, "
                        "dt=5 s, L=12,623,041 bins x A,E complex128; data = injected sum of all "
                        "binaries + Gaussian noise from the analytic A/E PSD",
            "binaries_per_gpu": int(B),
            "N_mix": {str(n): int(np.count_nonzero(Ns == n)) for n in np.unique(Ns)},
            "l2": "inputs larger than L2 (data + PSD: 606 MB); the GPU arm also writes 256 MB "
                  "before every timed step"}


def run_reference(args):
    """CPU reference arm: the reference's algorithm (the oracle port: NumPy
    waveform + the C likelihood loop, FP64) over the whole batch in every step
    on all host cores, on the same data as the GPU arm (host noise plus the
    injected sum of all binaries, built here by the oracle)."""
    p, Ns = draw_workload(args.binaries, args.seed)
    dA, dE, S = host_noise(args.seed)
    workers = os.cpu_count() or 1
    pool = CpuPool(dA, dE, S, workers)
    walls = []
    try:
        pool.inject(p, Ns)
        tasks = cpu_tasks(p, Ns, np.arange(p.shape[1]))
        for _ in range(max(0, args.warmup)):
            pool.run(tasks)
        for _ in range(max(1, args.steps)):
            walls.append(pool.run(tasks)[0])
    finally:
        pool.close()
    ms = float(np.mean(walls)) * 1e3
    v = args.binaries / (ms / 1e3)
    return {"metric": METRIC, "value": v, "unit": "binaries/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded binaries; injected sum + Gaussian noise "
                                    "from the analytic A/E PSD; the GPU arm's data)",
            "config": workload_config(args.binaries, Ns),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "binaries/s", "cores": int(workers), "kind": "port",
                             "sample": f"the whole {args.binaries}-binary batch in every step "
                                       f"(oracle: NumPy waveform + C get_ll), {workers} spawn "
                                       "workers, data resident in shared memory"},
            "e2e": {"value": v, "unit": "binaries/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--binaries", type=int, default=B_DEFAULT)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--cpu-workers", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fill-bench", action="store_true")
    ap.add_argument("--no-mcmc-bench", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="use the kernels' default launch shape instead of the autotuner's")
    ap.add_argument("--section", choices=["dropin", "pair", "fill"], default=None,
                    help="run one sub-benchmark alone (not the bench line)")
    args = ap.parse_args()
    if args.section == "dropin":
        print(json.dumps(dropin_section(args)), flush=True)
        return
    if args.section == "pair":
        print(json.dumps(pair_section(args)), flush=True)
        return
    if args.section == "fill":
        print(json.dumps(fill_section(args)), flush=True)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    out = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
