"""Launch-shape autotuner for the persistent waveform kernels.

The fused kernels take two launch parameters (``gbx_wave_args.tile`` and
``.blocks_per_sm``): samples per tile, which sets the binaries per block
(clamp(tile / N, 1, 16)) and the threads per binary of the likelihood
epilogue (256 / that), and the resident blocks per SM of the persistent grid.
Which shape is fastest depends on the N mix, the precision and the entry
point, so the tuner times every candidate on the caller's own batch (CUDA
events on the current stream, after one untimed launch) and keeps the
fastest.  Choices are cached per device, in memory and in a JSON file
(``GBX_AUTOTUNE_CACHE``; default ``~/.cache/gbgpu_gb300/autotune.json``), so a
workload is tuned once.  Results differ between shapes only by summation
order (a few ulps of the FP32 partial sums).

The reference has no counterpart (its kernels use one thread per binary).
"""

import json
import os
import threading

import numpy as np
import torch

TILES = (256, 512, 1024, 2048, 4096)
BLOCKS_PER_SM = (0, 2, 1)          # 0 = as many as fit


def _default_path():
    return os.environ.get("GBX_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "gbgpu_gb300",
                                       "autotune.json"))


def workload_key(kind, N, num_bin, precision, tdi2, nparams):
    """Key of a workload: entry point, N mix (each N with its count rounded
    to a power of two), precision, TDI generation and parameter count."""
    if np.ndim(N) == 0:
        mix = f"{int(N)}:{_pow2_bucket(num_bin)}"
    else:
        vals, counts = np.unique(np.asarray(N, dtype=np.int64), return_counts=True)
        mix = ",".join(f"{int(v)}:{_pow2_bucket(c)}" for v, c in zip(vals, counts))
    return f"{kind}|{mix}|{precision}|tdi2={int(bool(tdi2))}|np={int(nparams)}"


def _pow2_bucket(n):
    n = int(n)
    return 0 if n <= 0 else 1 << int(round(np.log2(n)))


class Autotuner:
    """Times candidate launch shapes and remembers the fastest per workload."""

    def __init__(self, path=None, candidates=None, reps=3):
        self.path = path if path is not None else _default_path()
        self.candidates = list(candidates) if candidates is not None else [
            (t, b) for t in TILES for b in BLOCKS_PER_SM]
        self.reps = int(reps)
        self._mem = {}
        self._lock = threading.Lock()
        self._loaded = False

    def _device_tag(self):
        p = torch.cuda.get_device_properties(torch.cuda.current_device())
        return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"

    def _load(self):
        if self._loaded:
            return
        self._loaded = True
        try:
            with open(self.path) as f:
                data = json.load(f)
            if isinstance(data, dict):
                self._mem.update({k: tuple(v) for k, v in data.items()})
        except (OSError, ValueError):
            pass

    def _save(self):
        try:
            os.makedirs(os.path.dirname(self.path) or ".", exist_ok=True)
            tmp = f"{self.path}.{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump({k: list(v) for k, v in self._mem.items()}, f, indent=0, sort_keys=True)
            os.replace(tmp, self.path)
        except OSError:
            pass

    def lookup(self, key):
        with self._lock:
            self._load()
            return self._mem.get(f"{self._device_tag()}|{key}")

    def tune(self, key, run):
        """``run(tile, blocks_per_sm)`` launches the kernel once on the current
        stream and raises RuntimeError for a shape that cannot launch.
        Returns the fastest (tile, blocks_per_sm) and caches it."""
        full = f"{self._device_tag()}|{key}"
        with self._lock:
            self._load()
            hit = self._mem.get(full)
        if hit is not None:
            return hit
        best, best_ms, timings = None, float("inf"), {}
        stream = torch.cuda.current_stream()
        for tile, bps in self.candidates:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            try:
                e0.record(stream)
                run(tile, bps)                       # first launch: builds the plan
                e1.record(stream)
            except RuntimeError:
                continue
            e1.synchronize()
            # long launches (the FP64 form of big batches) are timed once more
            reps = self.reps if e0.elapsed_time(e1) < 20.0 else 1
            e0.record(stream)
            for _ in range(reps):
                run(tile, bps)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / reps
            timings[(tile, bps)] = ms
            if ms < best_ms:
                best, best_ms = (tile, bps), ms
        if best is None:
            raise RuntimeError(f"no launch shape ran for workload {key}")
        with self._lock:
            self._mem[full] = best
            self._save()
        self.last_timings = timings
        return best


_TUNER = None


def default_tuner():
    global _TUNER
    if _TUNER is None:
        _TUNER = Autotuner()
    return _TUNER
