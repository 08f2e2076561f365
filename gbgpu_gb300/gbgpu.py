"""GBGPU class API on the GB300 kernels.

Mirrors gbgpu/gbgpu.py: ``GBGPUBase`` / ``GBGPU`` with ``run_wave`` (:108-316),
the output properties (:318-346, :542-578), ``get_ll`` (:580-735),
``fill_global_template`` (:737-837), ``generate_global_template`` (:839-878),
``inject_signal`` (:880-946), ``information_matrix`` (:957-1138) and the
extension hooks (:1140-1327).  Arrays live on the GPU as torch tensors; NumPy
inputs are accepted and copied to the device.  The waveform, likelihood and
template fill run in the CUDA kernels of ``libgbgpu_gb300.so``; ``get_ll`` and
``generate_global_template`` use fused kernels so the waveform never goes
through device memory, and the waveform attributes (``XYZf``, ``AETf``,
``start_inds`` ...) are then produced on first access.
"""

import abc
import ctypes
import os
import warnings

import numpy as np
import torch

from . import _native as nat
from .backend import get_backend
from .constants import YRSID_SI
from .orbits import EqualArmlengthOrbits, Orbits
from .utility import get_N

_PRECISIONS = {"fp64": nat.GBX_FP64, "mixed": nat.GBX_MIXED, "pair": nat.GBX_PAIR}
_TILE_MIN = 512       # default samples per tile of the fused kernels
_MAX_PACK = 16        # most binaries in one tile
_PLAN_CACHE = 64      # WavePlans kept per GBGPU object


def _is_pow2(n):
    return n >= 1 and (n & (n - 1)) == 0


def _as_tensor(x):
    """A torch view of an array from another library without a copy: objects
    with ``__cuda_array_interface__`` (CuPy, Numba, ...) or ``__dlpack__``;
    None for anything else (NumPy arrays, lists, scalars)."""
    if isinstance(x, (torch.Tensor, np.ndarray)):
        return None
    if hasattr(x, "__cuda_array_interface__"):
        return torch.as_tensor(x, device="cuda")
    if hasattr(x, "__dlpack__"):
        return torch.from_dlpack(x)
    return None


def _native(x):
    """``x`` itself, or a torch view of a foreign device array (see _as_tensor)."""
    t = _as_tensor(x)
    return x if t is None else t


def _to_device(x, dtype, device, non_blocking=False):
    """``x`` as a ``dtype`` tensor on ``device``: torch tensors, NumPy arrays
    and sequences, and device arrays of other libraries (CUDA array
    interface or DLPack, taken without a copy when dtype and device match).
    ``non_blocking`` queues a copy from pinned host memory on the current
    stream; only for callers that read their results back before returning."""
    if not isinstance(x, torch.Tensor):
        t = _as_tensor(x)
        if t is None:
            return torch.as_tensor(np.asarray(x), dtype=dtype, device=device)
        x = t
    nb = non_blocking and x.device.type == "cpu" and x.is_pinned() and x.dtype == dtype
    return x.to(device=device, dtype=dtype, non_blocking=nb)


_KEY_MULT = np.zeros((2, 0), dtype=np.uint64)


def _array_key(arr):
    """128-bit content key of an int64 array: two dot products with fixed
    random odd 64-bit multipliers, wrapping mod 2^64 (one vectorised pass; a
    cryptographic hash of a 200k-entry N array cost milliseconds per call)."""
    global _KEY_MULT
    n = arr.shape[0]
    if _KEY_MULT.shape[1] < n:
        rng = np.random.default_rng(0x5EED)
        m = max(n, 2 * _KEY_MULT.shape[1], 1024)
        _KEY_MULT = rng.integers(0, 2 ** 63, size=(2, m), dtype=np.uint64) * np.uint64(2) + \
            np.uint64(1)
    v = arr.view(np.uint64)
    with np.errstate(over="ignore"):
        return (int(np.dot(v, _KEY_MULT[0, :n])), int(np.dot(v, _KEY_MULT[1, :n])))


def _to_host(x):
    if not isinstance(x, torch.Tensor):
        t = _as_tensor(x)
        if t is None:
            return np.asarray(x)
        x = t
    return x.detach().cpu().numpy()


def plan_tiles(N_per_bin, tile=0):
    """Tile list for a batch of uneven N: binaries sorted by decreasing N,
    packed clamp(tile/N, 1, 16) per tile (tile 0 = 512 samples, the kernels'
    default).  Returns (order int32, tiles int32 (t, 4))."""
    Ns = np.asarray(N_per_bin, dtype=np.int64).reshape(-1)
    if Ns.size and (np.any(Ns < 32) or np.any(Ns & (Ns - 1))):
        raise NotImplementedError("per-binary N must be powers of two >= 32")
    order = np.argsort(-Ns, kind="stable").astype(np.int32)
    sortedN = Ns[order]
    tiles = []
    pos = 0
    for N in sorted(set(Ns.tolist()), reverse=True):
        cnt = int(np.count_nonzero(sortedN == N))
        P = min(_MAX_PACK, max(1, (tile or _TILE_MIN) // N))
        first = pos + np.arange(0, cnt, P)
        count = np.minimum(P, pos + cnt - first)
        lg = int(N).bit_length() - 1
        tiles.append(np.stack([np.full_like(first, lg), first, count, np.zeros_like(first)], 1))
        pos += cnt
    tiles = np.concatenate(tiles).astype(np.int32) if tiles else np.zeros((0, 4), np.int32)
    return order, tiles


class WavePlan:
    """Device-resident description of a batch (orbit tables, tiles, queue)."""

    def __init__(self, owner, N, T, precision, tdi2=False, nparams=9, tile=0, blocks_per_sm=0):
        self.owner = owner
        self.T = float(T)
        self.precision = precision
        self.tdi2 = int(tdi2)              # GBX_TDI2_BIT | GBX_TDI_UNEQUAL
        self.nparams = nparams
        self.tile = int(tile)
        self.blocks_per_sm = int(blocks_per_sm)
        dev = owner.device
        if np.ndim(N) == 0:
            self.uniform = True
            self.N = int(N)
            Ns = [self.N]
            self.order = self.tiles = None
            self.ntiles = 0
        else:
            self.uniform = False
            self.N = 0
            Ns_arr = np.asarray(N, dtype=np.int64).reshape(-1)
            order, tiles = plan_tiles(Ns_arr, self.tile)
            Ns = sorted(set(Ns_arr.tolist()))
            self.order = torch.as_tensor(order, device=dev)
            self.tiles = torch.as_tensor(tiles.reshape(-1), device=dev)
            self.ntiles = len(tiles)
        self.tables = {}
        for n in Ns:
            n = int(n)
            if not _is_pow2(n) or n < 32:
                raise NotImplementedError(f"N={n}: the CUDA path supports powers of two >= 32")
            self.tables[n.bit_length() - 1] = owner._orbit_table(n, self.T)
        self.queue = torch.zeros(1, dtype=torch.int32, device=dev) if not self.uniform else None
        self._ws = None

    def args(self, params, start_freq_ind=0, status=None, grad=False):
        """gbx_wave_args for this plan.  The struct holds references to the
        plan and to ``params`` so that the device buffers it points to (tile
        list, queue, workspace, orbit tables) live as long as it does."""
        a = nat.WaveArgs()
        a._keep = (self, params, status)
        a.params = params.data_ptr()
        a.num_bin = params.shape[1]
        a.nparams = params.shape[0]
        a.N = self.N
        a.precision = _PRECISIONS[self.precision]
        a.tdi2 = self.tdi2
        a.start_freq_ind = int(start_freq_ind)
        a.T = self.T
        a.armlength = float(self.owner.orbits.armlength)
        a.year = YRSID_SI
        for lg, t in self.tables.items():
            a.orbit[lg] = t.data_ptr()
        a.order = self.order.data_ptr() if self.order is not None else None
        a.tiles = self.tiles.data_ptr() if self.tiles is not None else None
        a.ntiles = self.ntiles
        a.queue = self.queue.data_ptr() if self.queue is not None else None
        a.status = status.data_ptr() if status is not None else None
        a.tile = self.tile
        a.blocks_per_sm = self.blocks_per_sm
        B = params.shape[1]
        need = (nat.lib().gbx_grad_workspace_bytes(B) if grad
                else nat.lib().gbx_wave_workspace_bytes(B))
        if need:
            if self._ws is None or self._ws.numel() * 16 < need:
                self._ws = torch.empty((need + 15) // 16, dtype=torch.complex128,
                                       device=self.owner.device)
            a.workspace = self._ws.data_ptr()
            a.workspace_bytes = self._ws.numel() * 16
        return a


class GBGPUBase(abc.ABC):
    """Batched FastGB Galactic-binary waveforms, likelihoods and templates.

    Args:
        orbits: object with ``get_pos(t, sc)``, ``armlength`` and ``t_base``
            (default: analytic ``EqualArmlengthOrbits``).
        force_backend: accepted for API compatibility; only the GPU exists.
        precision: ``"fp64"`` (plain form), ``"pair"`` (float-pair slow part,
            FFT and sums, within ~1e-9 of FP64) or ``"mixed"`` (FP64 phase,
            FP32 slow part and FFT) for the fused likelihood / fill kernels.
        unequal_arms: take each arm's length from the orbit at every sample
            (|P_j - P_i|) in the link transfer functions, antenna patterns and
            TDI delays, instead of the single ``orbits.armlength`` of the
            reference's equal-arm TDI (gbgpu.py:167-170); FP64 and pair forms.
            With equal arms both give the same windows.
        autotune: pick the fused kernels' launch shape (samples per tile,
            blocks per SM) by timing candidates on the first batch of each
            workload (cached per device); default from ``GBX_AUTOTUNE=1``.
    """

    NPARAMS = 9

    def __init__(self, orbits: Orbits = None, force_backend=None, precision="fp64", device=None,
                 autotune=None, unequal_arms=False):
        self._backend = get_backend(force_backend)
        self.unequal_arms = bool(unequal_arms)
        # launch shapes picked by timing (gbgpu_gb300.autotune); default from
        # the environment variable GBX_AUTOTUNE=1, else the kernels' defaults
        self.autotune = (os.environ.get("GBX_AUTOTUNE", "0") == "1") if autotune is None \
            else bool(autotune)
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {list(_PRECISIONS)}")
        self.precision = precision
        self.d_d = None
        self._tables = {}
        self._plans = {}
        self._shapes = {}
        self._n_last = None
        self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._lazy = None
        self._XYZf = self._AETf = self._start_inds = None
        self.orbits = orbits

    # ------------------------------------------------------------- plumbing
    @property
    def backend(self):
        """The backend method table (get_ll, fill_global, xp)."""
        return self._backend

    @property
    def xp(self):
        """The array module of the backend (torch here; CuPy/NumPy in the reference)."""
        return torch

    @classmethod
    def supported_backends(cls):
        """Backends this class runs on (gbgpu.py:72-74): the GB300 CUDA build only."""
        return ["gpu"]

    @property
    def get_ll_func(self):
        """The backend's native get_ll (gbgpu.py:76-79)."""
        return self.backend.get_ll

    @property
    def fill_global_func(self):
        """The backend's native fill_global (gbgpu.py:81-84)."""
        return self.backend.fill_global

    @property
    def orbits(self):
        """The spacecraft orbits (gbgpu.py:86-90)."""
        return self._orbits

    @orbits.setter
    def orbits(self, orbits):
        """Set the orbits; None selects the analytic EqualArmlengthOrbits (gbgpu.py:91-101)."""
        if orbits is None:
            self._orbits = EqualArmlengthOrbits()
        elif not (hasattr(orbits, "get_pos") and hasattr(orbits, "armlength")):
            raise ValueError("Input orbits must provide get_pos(t, sc), armlength and t_base")
        else:
            self._orbits = orbits
        self._orbits.configure(linear_interp_setup=True)
        self._tables = {}
        self._plans = {}

    @property
    def citation(self):
        """References to cite (gbgpu.py:103-106)."""
        return ("Katz et al. arXiv:2205.03461; Cornish & Littenberg arXiv:0704.1808; "
                "Robson et al. arXiv:1806.00500")

    def _orbit_table(self, N, T):
        key = (int(N), float(T))
        tab = self._tables.get(key)
        if tab is None:
            tm = np.linspace(0, T, num=N, endpoint=False)
            pos = np.stack([self.orbits.get_pos(tm, np.full(N, s, dtype=np.int32))
                            for s in (1, 2, 3)])
            pos_d = torch.as_tensor(np.ascontiguousarray(pos, dtype=np.float64), device=self.device)
            nbytes = nat.lib().gbx_orbit_table_bytes(N)
            tab = torch.empty((nbytes + 15) // 16 * 2, dtype=torch.float64, device=self.device)
            rc = nat.lib().gbx_orbit_table(ctypes.c_void_p(tab.data_ptr()),
                                          ctypes.c_void_p(pos_d.data_ptr()), int(N),
                                          float(self.orbits.armlength), nat.stream_handle())
            nat.check(rc, "gbx_orbit_table")
            self._tables[key] = tab
        return tab

    def _check_T(self, T):
        if T > np.max(self.orbits.t_base):
            raise ValueError(
                f"Observation time ({T}) is larger than length of time in orbital information "
                f"({np.max(self.orbits.t_base)})")

    def _plan(self, N, T, precision, tdi2, nparams, tile=0, blocks_per_sm=0, nkey=None,
              trusted=True):
        """WavePlan cache: tile schedules and orbit tables are built once per
        distinct (N or N-array contents, T, precision, tdi2, nparams, launch
        shape).  ``nkey`` is the N array's content key when the caller has it;
        with ``trusted=False`` it is the previous call's key for the same
        buffer, not yet verified against the contents, and serves only to find
        an existing plan: a new plan is always filed under the key of the
        contents it was built from."""
        # TDI code of the kernels: bit 0 TDI-2, bit 1 unequal arms
        tdi = (nat.GBX_TDI2_BIT if tdi2 else 0) | \
            (nat.GBX_TDI_UNEQUAL if getattr(self, "unequal_arms", False) else 0)
        if np.ndim(N) == 0:
            key = (int(N), float(T), precision, tdi, nparams, tile, blocks_per_sm)
        else:
            arr = np.ascontiguousarray(N, dtype=np.int64)
            rest = (arr.shape[0], float(T), precision, tdi, nparams, tile, blocks_per_sm)
            if nkey is None or (not trusted and (nkey,) + rest not in self._plans):
                nkey = _array_key(arr)
            key = (nkey,) + rest
        plan = self._plans.pop(key, None)
        if plan is None:
            # least recently used plans go first; a plan stays alive while any
            # gbx_wave_args built from it does (WavePlan.args keeps a reference)
            while len(self._plans) >= _PLAN_CACHE:
                self._plans.pop(next(iter(self._plans)))
            plan = WavePlan(self, N, T, precision, tdi, nparams, tile, blocks_per_sm)
        self._plans[key] = plan
        return plan

    def _params(self, base, add_args):
        if not isinstance(base, (list, tuple)):
            base = _native(base)
        if isinstance(base, (np.ndarray, torch.Tensor)) and base.ndim == 2 and not add_args:
            return _to_device(base, torch.float64, self.device).contiguous()
        cols = [torch.atleast_1d(_to_device(x, torch.float64, self.device)) for x in base]
        B = cols[0].shape[0]
        rows = [c.expand(B) if c.shape[0] == 1 and B > 1 else c for c in cols]
        for x in add_args:
            c = torch.atleast_1d(_to_device(x, torch.float64, self.device))
            rows.append(c.expand(B) if c.shape[0] == 1 and B > 1 else c)
        return torch.stack(rows).contiguous()

    def _resolve_N(self, N, amp, f0, T, args, oversample):
        if N is None:
            N = self.special_get_N(_to_host(amp), _to_host(f0), T, *[_to_host(a) for a in args],
                                   oversample=oversample)
            return int(np.max(N))
        if np.ndim(N) == 0:
            return int(N)
        return np.asarray(_to_host(N), dtype=np.int64).reshape(-1)

    # -------------------------------------------------------------- waveform
    def run_wave(self, amp, f0, fdot, fddot, phi0, iota, psi, lam, beta, *args, N=None,
                 T=4 * YRSID_SI, dt=10.0, oversample=1, tdi2=False, precision="fp64"):
        """Batched X/Y/Z and A/E/T windows (reference gbgpu/gbgpu.py:108-316).

        ``precision`` (not in the reference) is ``"fp64"`` (the plain form,
        default) or ``"pair"`` (float-pair arithmetic, within ~1e-10 of it);
        the FP32 ``"mixed"`` form is also accepted.
        """
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {list(_PRECISIONS)}")
        N_obs = int(T / dt)
        T = N_obs * dt
        self._check_T(T)
        add_args = self.prepare_additional_args(*args) if len(args) else ()
        N = self._resolve_N(N, amp, f0, T, args, oversample)
        if np.ndim(N) != 0:
            raise NotImplementedError("run_wave takes one N per call (as the reference)")
        params = self._params((amp, f0, fdot, fddot, phi0, iota, psi, lam, beta), add_args)
        self._wave_from_params(params, N, T, tdi2, precision)

    def _wave_from_params(self, params, N, T, tdi2, precision="fp64"):
        B = params.shape[1]
        self.num_bin = B
        self.N = N
        self.df = 1 / T
        plan = self._plan(N, T, precision, tdi2, params.shape[0])
        XYZ = torch.empty((B, 3, N), dtype=torch.complex128, device=self.device)
        AET = torch.empty((B, 3, N), dtype=torch.complex128, device=self.device)
        start = torch.empty(B, dtype=torch.int32, device=self.device)
        if B:
            a = plan.args(params)
            rc = nat.lib().gbx_waveform(ctypes.byref(a), nat.ptr(XYZ), nat.ptr(AET), nat.ptr(start),
                                        nat.stream_handle())
            nat.check(rc, "gbx_waveform")
        self._lazy = None
        self._XYZf, self._AETf = XYZ, AET
        self._start_inds = start.to(torch.int64)

    def _materialize(self):
        if self._lazy is not None:
            params, N, T, tdi2 = self._lazy
            self._lazy = None
            if np.ndim(N) != 0:
                raise RuntimeError("waveform arrays are only defined for a single N per batch")
            self._wave_from_params(params, N, T, tdi2)

    @property
    def XYZf(self):
        """X, Y, Z windows (B, 3, N), computed on first access after a fused call."""
        self._materialize()
        return self._XYZf

    @XYZf.setter
    def XYZf(self, v):
        self._XYZf = v

    @property
    def AETf(self):
        """A, E, T windows (B, 3, N), computed on first access after a fused call."""
        self._materialize()
        return self._AETf

    @AETf.setter
    def AETf(self, v):
        self._AETf = v

    @property
    def start_inds(self):
        """First frequency bin of each window (B,), bit-exact with the reference (gbgpu.py:296-307)."""
        self._materialize()
        return self._start_inds

    @start_inds.setter
    def start_inds(self, v):
        self._start_inds = v

    @property
    def kmin(self):
        """Alias of start_inds."""
        return self.start_inds

    @property
    def X_out(self):
        """X window, point-major flat (index i*B + b) (gbgpu.py:318-322)."""
        return self.XYZf[:, 0].T.flatten()

    @property
    def Y_out(self):
        """Y window, point-major flat (gbgpu.py:323-327)."""
        return self.XYZf[:, 1].T.flatten()

    @property
    def Z_out(self):
        """Z window, point-major flat (gbgpu.py:328-332)."""
        return self.XYZf[:, 2].T.flatten()

    @property
    def A_out(self):
        """A window, point-major flat (gbgpu.py:333-337)."""
        return self.AETf[:, 0].T.flatten()

    @property
    def E_out(self):
        """E window, point-major flat (gbgpu.py:338-342)."""
        return self.AETf[:, 1].T.flatten()

    @property
    def T_out(self):
        """T window, point-major flat (gbgpu.py:343-346)."""
        return self.AETf[:, 2].T.flatten()

    @property
    def A(self):
        """A windows (B, N) (gbgpu.py:542-546)."""
        return self.AETf[:, 0]

    @property
    def E(self):
        """E windows (B, N) (gbgpu.py:547-551)."""
        return self.AETf[:, 1]

    @property
    def T(self):
        """T windows (B, N) (gbgpu.py:552-556)."""
        return self.AETf[:, 2]

    @property
    def X(self):
        """X windows (B, N) (gbgpu.py:557-561)."""
        return self.XYZf[:, 0]

    @property
    def Y(self):
        """Y windows (B, N) (gbgpu.py:562-566)."""
        return self.XYZf[:, 1]

    @property
    def Z(self):
        """Z windows (B, N) (gbgpu.py:567-571)."""
        return self.XYZf[:, 2]

    @property
    def freqs(self):
        """Frequencies of the window bins, (start_inds + arange(N)) df, (B, N) (gbgpu.py:572-578)."""
        k = torch.arange(self.N, device=self.device)[None, :] + self.start_inds[:, None]
        return k.to(torch.float64) * self.df

    # ------------------------------------------------------------ likelihood
    def _prepare_data(self, data, psd, data_index, noise_index, num_bin):
        data = [_native(x) for x in data]
        psd = [_native(x) for x in psd]
        data_index = None if data_index is None else _native(data_index)
        noise_index = None if noise_index is None else _native(noise_index)
        if not isinstance(data[0], (torch.Tensor, np.ndarray)):
            raise TypeError("Make sure the data arrays are torch tensors (or NumPy arrays).")
        d0 = data[0]
        if d0.ndim == 1:
            if data_index is not None:
                raise ValueError("If inputing 1D data, cannot use data_index kwarg.")
            if noise_index is not None:
                raise ValueError("If inputing 1D data, cannot use noise_index kwarg.")
            data_length = d0.shape[0]
        elif d0.ndim == 2:
            data_length = d0.shape[1]
        else:
            raise ValueError("data must be 1-D or 2-D")
        dd = [_to_device(x, torch.complex128, self.device).reshape(-1).contiguous() for x in data]
        pp = [_to_device(x, torch.float64, self.device).reshape(-1).contiguous() for x in psd]
        if data_index is None:
            data_index = torch.zeros(num_bin, dtype=torch.int32, device=self.device)
        if noise_index is None:
            noise_index = torch.zeros(num_bin, dtype=torch.int32, device=self.device)
        # reference checks (gbgpu.py:681-686)
        assert len(data_index) == num_bin
        assert len(data_index) == len(noise_index)
        assert str(data_index.dtype).endswith("int32")
        assert str(noise_index.dtype).endswith("int32")
        data_index = _to_device(data_index, torch.int32, self.device).contiguous()
        noise_index = _to_device(noise_index, torch.int32, self.device).contiguous()
        return dd, pp, data_length, data_index, noise_index

    def _launch_shape(self, kind, N, B, precision, tdi2, nparams, run, nkey=None, trusted=True):
        """(tile, blocks_per_sm) for this workload: the autotuner's choice when
        autotuning is on (timing ``run`` on the first call), else defaults.
        An unverified ``nkey`` (``trusted=False``) only looks up a cached
        shape; a shape tuned now is filed under the contents' own key."""
        if not self.autotune:
            return 0, 0
        if nkey is None:
            nkey = int(N) if np.ndim(N) == 0 else _array_key(np.ascontiguousarray(N, dtype=np.int64))
        ck = (kind, nkey, int(B), precision, bool(tdi2), int(nparams))
        shape = self._shapes.get(ck)
        if shape is None and not trusted and np.ndim(N) != 0:
            nkey = _array_key(np.ascontiguousarray(N, dtype=np.int64))
            ck = (kind, nkey, int(B), precision, bool(tdi2), int(nparams))
            shape = self._shapes.get(ck)
        if shape is None:
            from .autotune import default_tuner, workload_key
            shape = default_tuner().tune(workload_key(kind, N, B, precision, tdi2, nparams), run)
            self._shapes[ck] = shape
        return shape

    @staticmethod
    def _ll_args(dd, pp, data_length, data_index, noise_index, T):
        la = nat.LLArgs()
        la._keep = (dd, pp, data_index, noise_index)     # the struct holds raw pointers
        la.A_data, la.E_data = dd[0].data_ptr(), dd[1].data_ptr()
        la.A_psd, la.E_psd = pp[0].data_ptr(), pp[1].data_ptr()
        la.data_length = int(data_length)
        la.num_data = int(dd[0].numel() // data_length)
        la.num_psd = int(pp[0].numel() // data_length)
        la.data_index = data_index.data_ptr()
        la.noise_index = noise_index.data_ptr()
        la.df = 1.0 / T
        return la

    def _fused_ll(self, params, N, T, tdi2, dd, pp, data_length, data_index, noise_index,
                  start_freq_ind, precision):
        B = params.shape[1]
        d_h = torch.empty(B, dtype=torch.complex128, device=self.device)
        h_h = torch.empty(B, dtype=torch.complex128, device=self.device)
        if B == 0:
            return d_h, h_h
        la = self._ll_args(dd, pp, data_length, data_index, noise_index, T)
        nparams = params.shape[0]
        # content key of a per-binary N array (plan cache, launch shape); see _n_key
        arr, nkey, verify = None, None, False
        if np.ndim(N) != 0:
            arr = np.ascontiguousarray(N, dtype=np.int64)
            nkey, verify = self._n_key(arr)

        def run(tile, bps):
            plan = self._plan(N, T, precision, tdi2, nparams, tile, bps, nkey=nkey,
                              trusted=not verify)
            a = plan.args(params, start_freq_ind, self._status)
            rc = nat.lib().gbx_waveform_ll(ctypes.byref(a), ctypes.byref(la), nat.ptr(d_h),
                                           nat.ptr(h_h), nat.stream_handle())
            nat.check(rc, "gbx_waveform_ll")

        shape = self._launch_shape("ll", N, B, precision, tdi2, nparams, run, nkey=nkey,
                                   trusted=not verify)
        self._status.zero_()
        run(*shape)
        if verify:
            # the full key, computed while the kernel runs; if the array changed
            # in place, the launch is repeated with the right plan (same stream:
            # its outputs replace the first launch's before anyone reads them)
            full = _array_key(arr)
            self._n_last = self._n_last[:3] + (full,)
            verify = False
            if full != nkey:
                nkey = full
                shape = self._launch_shape("ll", N, B, precision, tdi2, nparams, run, nkey=nkey)
                self._status.zero_()
                run(*shape)
        return d_h, h_h

    def _n_key(self, arr):
        """(content key, needs verification) of an int64 N array.  A buffer
        that comes back at the same address with the same length and the same
        64 sampled entries reuses the previous call's key, to be verified
        against the full key after the launch (the full key costs a pass over
        the array on the host, which then overlaps the kernel); any other
        array gets its full key now."""
        n = arr.shape[0]
        sample = arr[::max(1, n // 64)].tobytes()
        last = self._n_last
        if last is not None and last[0] == arr.ctypes.data and last[1] == n and last[2] == sample:
            return last[3], True
        key = _array_key(arr)
        self._n_last = (arr.ctypes.data, n, sample, key)
        return key, False

    def _check_status(self):
        st = int(self._status.item())
        if st & nat.GBX_FLAG_INDEX:
            raise ValueError("a data/noise/group index is out of range")
        if st & nat.GBX_FLAG_WINDOW:
            warnings.warn("some template windows extend past the data arrays; "
                          "those bins were left out of the inner products")
        if st & nat.GBX_FLAG_TILE:
            raise RuntimeError("malformed tile schedule")

    def get_ll(self, params, data, psd, phase_marginalize=False, start_freq_ind=0,
               data_index=None, noise_index=None, **kwargs):
        """Batched log-likelihood -1/2 (<d|d> + <h|h> - 2 <d|h>) (gbgpu.py:580-735).

        ``params`` is (nparams, B).  Extra keywords go to the waveform
        (N, T, dt, oversample, tdi2) plus ``precision`` ("fp64" / "mixed").
        ``N`` may also be an array with one power-of-two N per binary; the
        batch then runs as one persistent work-queue launch.
        """
        if self.d_d is None:
            raise ValueError(
                "self.d_d attribute must be set before computing log-Likelihood. This attribute "
                "is the data with data inner product (<d|d>).")
        precision = kwargs.pop("precision", self.precision)
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {list(_PRECISIONS)}")
        N = kwargs.pop("N", None)
        T = kwargs.pop("T", 4 * YRSID_SI)
        dt = kwargs.pop("dt", 10.0)
        oversample = kwargs.pop("oversample", 1)
        tdi2 = kwargs.pop("tdi2", False)
        if kwargs:
            raise TypeError(f"unexpected keyword arguments {list(kwargs)}")
        T = int(T / dt) * dt
        self._check_T(T)
        params = params if isinstance(params, (list, tuple)) else _native(params)
        if isinstance(params, (np.ndarray, torch.Tensor)) and params.ndim == 2 and \
                params.shape[0] == self.NPARAMS:
            # get_ll reads the likelihood back before returning
            prm = _to_device(params, torch.float64, self.device, non_blocking=True).contiguous()
            base = [params[0], params[1]]
            extra = [params[i] for i in range(9, self.NPARAMS)]
            if extra:
                self.prepare_additional_args(*extra)
            if N is None:
                N = self._resolve_N(N, base[0], base[1], T, extra, oversample)
            elif np.ndim(N) != 0:
                N = np.asarray(_to_host(N), dtype=np.int64).reshape(-1)
            else:
                N = int(N)
        else:
            p = list(params)
            base, extra = p[:9], p[9:]
            add_args = self.prepare_additional_args(*extra) if extra else ()
            N = self._resolve_N(N, base[0], base[1], T, extra, oversample)
            prm = self._params(base, add_args)
        B = prm.shape[1]
        self.num_bin = B
        self.N = N
        self.df = df = 1 / T
        dd, pp, L, di, ni = self._prepare_data(data, psd, data_index, noise_index, B)
        d_h, h_h = self._fused_ll(prm, N, T, tdi2, dd, pp, L, di, ni, start_freq_ind, precision)
        self._lazy = (prm, N, T, tdi2)
        if phase_marginalize:
            self.non_marg_d_h = d_h.cpu().numpy().copy()
            d_h = torch.abs(d_h).to(torch.complex128)
        self.h_h = h_h
        self.d_h = d_h
        # the reference's order, -1/2 (d_d + h_h - 2 d_h) (gbgpu.py:728); a
        # scalar d_d enters as a kernel argument, not a device copy
        d_d = float(self.d_d) if np.ndim(_to_host(self.d_d)) == 0 else \
            torch.as_tensor(self.d_d, device=self.device)
        like = -1.0 / 2.0 * (d_d + h_h - 2 * d_h).real
        out = like.cpu().numpy()
        self._check_status()
        return out

    def get_ll_grad(self, params, data, psd, start_freq_ind=0, data_index=None,
                    noise_index=None, **kwargs):
        """Log-likelihood and its gradient in one fused launch (mixed form).

        Returns ``(like, grad)``: NumPy ``(B,)`` and ``(NPARAMS, B)`` with
        ``grad[k, b] = d like[b] / d params[k, b]`` for amp, f0, fdot, fddot,
        phi0, iota, psi, lam, beta (and, for GBGPUThirdBody, A2, varpi, e2,
        P2, T2).  No counterpart in the reference (its derivatives are finite
        differences, gbgpu.py:957-1138).  Set ``return_tensors=True`` to get
        device tensors instead.
        """
        like, grad = self._ll_grad_tensors(params, data, psd, start_freq_ind, data_index,
                                           noise_index, **kwargs)
        if kwargs.get("return_tensors"):
            return like, grad
        return like.cpu().numpy(), grad.cpu().numpy()

    def _ll_grad_tensors(self, params, data, psd, start_freq_ind=0, data_index=None,
                         noise_index=None, **kwargs):
        if self.d_d is None:
            raise ValueError("self.d_d attribute must be set before computing log-Likelihood.")
        kwargs.pop("return_tensors", None)
        kwargs.pop("precision", None)
        N = kwargs.pop("N", None)
        T = kwargs.pop("T", 4 * YRSID_SI)
        dt = kwargs.pop("dt", 10.0)
        oversample = kwargs.pop("oversample", 1)
        tdi2 = kwargs.pop("tdi2", False)
        if kwargs:
            raise TypeError(f"unexpected keyword arguments {list(kwargs)}")
        T = int(T / dt) * dt
        self._check_T(T)
        prm = _to_device(params, torch.float64, self.device).detach().contiguous()
        npar = self.NPARAMS
        if prm.ndim != 2 or prm.shape[0] != npar:
            raise ValueError(f"params must be ({npar}, B)")
        extra = [prm[i] for i in range(9, npar)]
        if extra:
            self.prepare_additional_args(*extra)
        if N is None:
            N = self._resolve_N(N, prm[0], prm[1], T, extra, oversample)
        elif np.ndim(N) != 0:
            N = np.asarray(_to_host(N), dtype=np.int64).reshape(-1)
        else:
            N = int(N)
        B = prm.shape[1]
        self.num_bin, self.N, self.df = B, N, 1 / T
        dd, pp, L, di, ni = self._prepare_data(data, psd, data_index, noise_index, B)
        d_h = torch.empty(B, dtype=torch.complex128, device=self.device)
        h_h = torch.empty(B, dtype=torch.complex128, device=self.device)
        grad = torch.zeros((npar, B), dtype=torch.float64, device=self.device)
        if B:
            la = self._ll_args(dd, pp, L, di, ni, T)

            def run(tile, bps):
                plan = self._plan(N, T, "mixed", tdi2, npar, tile, bps)
                a = plan.args(prm, start_freq_ind, self._status, grad=True)
                rc = nat.lib().gbx_waveform_ll_grad(ctypes.byref(a), ctypes.byref(la),
                                                    nat.ptr(d_h), nat.ptr(h_h), nat.ptr(grad),
                                                    nat.stream_handle())
                nat.check(rc, "gbx_waveform_ll_grad")

            shape = self._launch_shape("grad", N, B, "mixed", tdi2, npar, run)
            self._status.zero_()
            run(*shape)
        self._lazy = (prm, N, T, tdi2)
        self.d_h, self.h_h = d_h, h_h
        d_d = torch.as_tensor(self.d_d, device=self.device)
        like = -0.5 * (d_d + h_h.real - 2 * d_h.real)
        return like, grad

    def swap_likelihood(self, params_old, params_new, data, psd, start_freq_ind=0,
                        data_index=None, noise_index=None, return_tensor=False, grad=False,
                        **kwargs):
        """Change of log-likelihood when source ``params_old[:, j]`` is replaced by
        ``params_new[:, j]`` (no counterpart in this version of the reference).

        ``data`` holds residuals r = d - (current sum of sources), one row per
        walker selected by ``data_index``; with Dh = h_new - h_old,
        ``dlogL_j = Re<r|Dh> - <Dh|Dh>/2`` over the union of both windows, in
        the inner product of the reference's likelihood.  Keywords as in
        ``get_ll`` (N must be a single power of two; ``precision``).

        With ``grad=True`` returns ``(dlogL, grad)``, ``grad[k, j] = d dlogL_j /
        d params_new[k, j]`` (= Re<r + h_old - h_new | d h_new>, the likelihood
        gradient at the proposal against r + h_old), both in the mixed form.
        """
        precision = kwargs.pop("precision", "mixed" if grad else self.precision)
        if grad and precision != "mixed":
            raise ValueError("swap gradients are computed in the mixed form only")
        N = kwargs.pop("N", None)
        T = kwargs.pop("T", 4 * YRSID_SI)
        dt = kwargs.pop("dt", 10.0)
        oversample = kwargs.pop("oversample", 1)
        tdi2 = kwargs.pop("tdi2", False)
        if kwargs:
            raise TypeError(f"unexpected keyword arguments {list(kwargs)}")
        T = int(T / dt) * dt
        self._check_T(T)
        po = _to_device(params_old, torch.float64, self.device)
        pn = _to_device(params_new, torch.float64, self.device)
        if po.shape != pn.shape or po.ndim != 2 or po.shape[0] != self.NPARAMS:
            raise ValueError(f"params_old / params_new must both be ({self.NPARAMS}, B)")
        B = po.shape[1]
        if N is None:
            N = max(self._resolve_N(None, po[0], po[1], T, [po[i] for i in range(9, self.NPARAMS)],
                                    oversample),
                    self._resolve_N(None, pn[0], pn[1], T, [pn[i] for i in range(9, self.NPARAMS)],
                                    oversample))
        if np.ndim(N) != 0:
            raise NotImplementedError("swap_likelihood takes one N per call")
        N = int(N)
        prm = torch.stack([po, pn], dim=2).reshape(self.NPARAMS, 2 * B).contiguous()
        di = None if data_index is None else _to_device(data_index, torch.int32, self.device)
        ni = None if noise_index is None else _to_device(noise_index, torch.int32, self.device)
        di2 = None if di is None else di.repeat_interleave(2).contiguous()
        ni2 = None if ni is None else ni.repeat_interleave(2).contiguous()
        dd, pp, L, di2, ni2 = self._prepare_data(data, psd, di2, ni2, 2 * B)
        out = torch.empty(B, dtype=torch.float64, device=self.device)
        gout = torch.zeros((self.NPARAMS, B), dtype=torch.float64, device=self.device) if grad else None
        if B:
            plan = self._plan(N, T, precision, tdi2, self.NPARAMS)
            self._status.zero_()
            a = plan.args(prm, start_freq_ind, self._status, grad=grad)
            la = nat.LLArgs()
            la.A_data, la.E_data = dd[0].data_ptr(), dd[1].data_ptr()
            la.A_psd, la.E_psd = pp[0].data_ptr(), pp[1].data_ptr()
            la.data_length = int(L)
            la.num_data = int(dd[0].numel() // L)
            la.num_psd = int(pp[0].numel() // L)
            la.data_index = di2.data_ptr()
            la.noise_index = ni2.data_ptr()
            la.df = 1.0 / T
            if grad:
                rc = nat.lib().gbx_swap_ll_grad(ctypes.byref(a), ctypes.byref(la), nat.ptr(out),
                                                nat.ptr(gout), nat.stream_handle())
                nat.check(rc, "gbx_swap_ll_grad")
            else:
                rc = nat.lib().gbx_swap_ll(ctypes.byref(a), ctypes.byref(la), nat.ptr(out),
                                           nat.stream_handle())
                nat.check(rc, "gbx_swap_ll")
        if return_tensor:
            return (out, gout) if grad else out
        res = out.cpu().numpy()
        self._check_status()
        return (res, gout.cpu().numpy()) if grad else res

    # --------------------------------------------------------- global fill
    def fill_global_template(self, group_index, templates, A, E, start_inds, N=None,
                             start_freq_ind=0, mode="atomic"):
        """Sum waveforms into templates[g, 0:2] (gbgpu.py:737-837), in place.

        Channels 0 and 1 of ``templates`` are overwritten with the new sums,
        as in the reference; other channels are untouched.  ``mode="atomic"``
        adds with FP64 atomics (summation order varies between runs, as on the
        reference's GPU backend); ``mode="deterministic"`` sorts the binaries
        by (group, start) and gathers every output bin in that order, giving
        identical bits on every run.
        """
        templates = _native(templates)
        if mode not in ("atomic", "deterministic"):
            raise ValueError("mode must be 'atomic' or 'deterministic'")
        total_groups, nchannels, data_length = templates.shape
        num_bin = len(group_index)
        if nchannels < 2:
            raise ValueError("Calculates for A and E channels.")
        elif nchannels > 2:
            warnings.warn("Only calculating A and E channels here currently.")
        if not isinstance(templates, (torch.Tensor, np.ndarray)):
            raise TypeError("Make sure the data arrays are the same type as template arrays.")
        host_out = isinstance(templates, np.ndarray)
        tt = _to_device(templates, torch.complex128, self.device)
        work = tt if tt.is_contiguous() else tt.contiguous()
        gi = _to_device(group_index, torch.int32, self.device).contiguous()
        si = (_to_device(start_inds, torch.int64, self.device) - start_freq_ind).to(torch.int32).contiguous()
        A = _to_device(A, torch.complex128, self.device)
        E = _to_device(E, torch.complex128, self.device)
        if A.ndim > 2 or E.ndim > 2:
            raise ValueError("A_in, E_in have maximum allowable dimension of 2.")
        elif A.ndim == 2:
            N = A.shape[1]
            assert E.ndim == 2
            if A.stride() != E.stride():
                A, E = A.contiguous(), E.contiguous()
            tsb, tsi = A.stride()
        elif A.ndim == 1:
            if N is None:
                raise ValueError("If providing a 1D flattened array for A and E, the N kwarg "
                                 "also needs to be provided.")
            A, E = A.contiguous(), E.contiguous()
            tsi, tsb = num_bin, 1
        if mode == "deterministic":
            self._fill_det(work, gi, si, A, E, int(N), int(tsi), int(tsb))
            self._finish_fill(templates, tt, work, host_out)
            return
        work[:, 0:2].zero_()
        self._status.zero_()
        if num_bin:
            rc = nat.lib().gbx_fill_global_ex(
                ctypes.c_void_p(work[0, 0].data_ptr()), ctypes.c_void_p(work[0, 1].data_ptr()),
                ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(E.data_ptr()),
                ctypes.c_void_p(si.data_ptr()), int(N), int(num_bin),
                ctypes.c_void_p(gi.data_ptr()), int(data_length), int(total_groups),
                int(nchannels * data_length), int(tsi), int(tsb),
                ctypes.c_void_p(self._status.data_ptr()), nat.stream_handle())
            nat.check(rc, "gbx_fill_global_ex")
        self._finish_fill(templates, tt, work, host_out)

    def _fill_det(self, work, gi, si, A, E, N, tsi, tsb):
        """Sorted gather into channels 0/1 of ``work`` (G, nch, L), in place."""
        G, nch, L = work.shape
        B = gi.shape[0]
        if B and (int(gi.min()) < 0 or int(gi.max()) >= G):
            raise ValueError("group_index out of range")
        key = (gi.to(torch.int64) << 32) | (si.to(torch.int64) + (1 << 31))
        order = torch.argsort(key, stable=True).to(torch.int32).contiguous()
        first = torch.zeros(G + 1, dtype=torch.int32, device=self.device)
        if B:
            first[1:] = torch.cumsum(torch.bincount(gi.to(torch.int64), minlength=G), 0).to(torch.int32)
        rc = nat.lib().gbx_fill_global_det(
            ctypes.c_void_p(work[0, 0].data_ptr()), ctypes.c_void_p(work[0, 1].data_ptr()),
            ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(E.data_ptr()),
            ctypes.c_void_p(si.data_ptr()), int(N), int(B), ctypes.c_void_p(order.data_ptr()),
            ctypes.c_void_p(first.data_ptr()), int(G), int(L), int(nch * L), int(tsi), int(tsb),
            nat.stream_handle())
        nat.check(rc, "gbx_fill_global_det")

    def _finish_fill(self, templates, tt, work, host_out):
        if work is not tt:
            tt.copy_(work)
        if host_out:
            templates[...] = tt.cpu().numpy()
        elif tt is not templates:
            templates.copy_(tt)
        if int(self._status.item()) & nat.GBX_FLAG_INDEX:
            raise ValueError("group_index out of range")

    def generate_global_template(self, params, group_index, templates, start_freq_ind=0,
                                 **kwargs):
        """Waveforms straight into templates (gbgpu.py:839-878), fused on the GPU.

        ``params`` is (B, nparams), transposed relative to ``get_ll``.  With
        ``sort=True`` (atomic mode, one N) the binaries are launched in order
        of (group, carrier bin), so that a tile holds frequency neighbours of
        one group and the kernel adds their overlapping windows once (fewer
        atomics in dense bands; the sum is the same up to FP64 rounding).
        """
        templates = _native(templates)
        precision = kwargs.pop("precision", self.precision)
        fill_mode = kwargs.pop("fill_mode", "atomic")
        sort = bool(kwargs.pop("sort", False))
        if fill_mode not in ("atomic", "deterministic"):
            raise ValueError("fill_mode must be 'atomic' or 'deterministic'")
        N = kwargs.pop("N", None)
        T = kwargs.pop("T", 4 * YRSID_SI)
        dt = kwargs.pop("dt", 10.0)
        oversample = kwargs.pop("oversample", 1)
        tdi2 = kwargs.pop("tdi2", False)
        T = int(T / dt) * dt
        self._check_T(T)
        pT = _to_device(params, torch.float64, self.device).T
        base, extra = [pT[i] for i in range(9)], [pT[i] for i in range(9, pT.shape[0])]
        add_args = self.prepare_additional_args(*extra) if extra else ()
        N = self._resolve_N(N, base[0], base[1], T, extra, oversample)
        prm = self._params(base, add_args)
        B = prm.shape[1]
        self.num_bin, self.N, self.df = B, N, 1 / T
        total_groups, nchannels, data_length = templates.shape
        if nchannels < 2:
            raise ValueError("Calculates for A and E channels.")
        host_out = isinstance(templates, np.ndarray)
        tt = _to_device(templates, torch.complex128, self.device)
        work = tt if tt.is_contiguous() else tt.contiguous()
        gi = _to_device(group_index, torch.int32, self.device).contiguous()
        if fill_mode == "deterministic":
            # waveform windows first (A/E/T, (B, 3, N)), then the sorted gather
            if np.ndim(N) != 0:
                raise NotImplementedError("deterministic fill takes one N per call")
            AET = torch.empty((B, 3, int(N)), dtype=torch.complex128, device=self.device)
            start = torch.empty(B, dtype=torch.int32, device=self.device)
            if B:
                plan = self._plan(N, T, precision, tdi2, prm.shape[0])
                a = plan.args(prm, start_freq_ind, self._status)
                rc = nat.lib().gbx_waveform(ctypes.byref(a), None, nat.ptr(AET), nat.ptr(start),
                                            nat.stream_handle())
                nat.check(rc, "gbx_waveform")
            self._fill_det(work, gi, start, AET[:, 0], AET[:, 1], int(N), 1, 3 * int(N))
            self._lazy = (prm, N, T, tdi2)
            self._finish_fill(templates, tt, work, host_out)
            return
        work[:, 0:2].zero_()
        self._status.zero_()
        if B:
            plan = self._plan(N, T, precision, tdi2, prm.shape[0], self._fill_tile(N, sort))
            a = plan.args(prm, start_freq_ind, self._status)
            if sort:
                self._fill_order(a, prm, gi, T, N)
            rc = nat.lib().gbx_waveform_fill(
                ctypes.byref(a), ctypes.c_void_p(work[0, 0].data_ptr()),
                ctypes.c_void_p(work[0, 1].data_ptr()), ctypes.c_void_p(gi.data_ptr()),
                int(total_groups), int(data_length), int(nchannels * data_length),
                nat.stream_handle())
            nat.check(rc, "gbx_waveform_fill")
        self._lazy = (prm, N, T, tdi2)
        self._finish_fill(templates, tt, work, host_out)

    def add_to_templates(self, params, group_index, templates, start_freq_ind=0, **kwargs):
        """Add waveforms into templates without zeroing them first (no
        counterpart in the reference, whose fill always overwrites).

        ``params`` is (nparams, B) on the device; ``templates`` is either a
        contiguous (G, nch, L) complex128 CUDA tensor (channels 0 and 1 are
        A and E) or a pair ``(A, E)`` of contiguous (G, L) tensors; they are
        updated in place with FP64 atomics.  Nothing here synchronises or
        copies from the host once the plan for (N, T, precision) exists, so the
        call can be captured in a CUDA graph.
        """
        precision = kwargs.pop("precision", self.precision)
        N = int(kwargs.pop("N"))
        T = kwargs.pop("T", 4 * YRSID_SI)
        dt = kwargs.pop("dt", 10.0)
        tdi2 = kwargs.pop("tdi2", False)
        sort = bool(kwargs.pop("sort", False))
        if kwargs:
            raise TypeError(f"unexpected keyword arguments {list(kwargs)}")
        T = int(T / dt) * dt
        if isinstance(templates, (tuple, list)):
            tA, tE = templates
            if not (tA.is_cuda and tE.is_cuda and tA.is_contiguous() and tE.is_contiguous()
                    and tA.shape == tE.shape and tA.ndim == 2):
                raise TypeError("(A, E) templates must be contiguous (G, L) CUDA tensors")
            G, L = tA.shape
            pA, pE, gstride = tA.data_ptr(), tE.data_ptr(), L
        else:
            if not (isinstance(templates, torch.Tensor) and templates.is_cuda
                    and templates.is_contiguous()):
                raise TypeError("templates must be a contiguous CUDA tensor")
            G, nch, L = templates.shape
            pA, pE, gstride = templates[0, 0].data_ptr(), templates[0, 1].data_ptr(), nch * L
        B = params.shape[1]
        if B == 0:
            return
        plan = self._plan(N, T, precision, tdi2, params.shape[0], self._fill_tile(N, sort))
        a = plan.args(params, start_freq_ind, self._status)
        if sort:
            self._fill_order(a, params, group_index, T, N)
        rc = nat.lib().gbx_waveform_fill(
            ctypes.byref(a), ctypes.c_void_p(pA), ctypes.c_void_p(pE),
            ctypes.c_void_p(group_index.data_ptr()), int(G), int(L), int(gstride),
            nat.stream_handle())
        nat.check(rc, "gbx_waveform_fill")

    @staticmethod
    def _fill_tile(N, sort):
        """Samples per tile of a fill: sorted fills pack up to 16 binaries (at
        most 4096 samples) so that neighbours share a tile; else the default."""
        if not sort or np.ndim(N) != 0:
            return 0
        return int(min(16 * int(N), 4096))

    @staticmethod
    def _fill_order(a, prm, gi, T, N):
        """Launch order by (group, carrier bin rint(f0 T)) for a fill of one N
        (device sort; the order tensor is kept alive with the arguments)."""
        if np.ndim(N) != 0:
            raise NotImplementedError("sorted fills take one N per call")
        key = gi.to(torch.int64) * (1 << 40) + torch.round(prm[1] * T).to(torch.int64)
        order = torch.argsort(key).to(torch.int32).contiguous()
        a.order = order.data_ptr()
        a._keep = tuple(a._keep) + (order,)

    # ------------------------------------------------------------- injection
    def inject_signal(self, *args, fmax=None, T=4.0 * YRSID_SI, dt=10.0, **kwargs):
        """Binary 0 placed on a 0..fmax grid, as NumPy (A, E) (gbgpu.py:880-946)."""
        if fmax is None:
            fmax = 1 / (2 * dt)
        self._check_T(T)
        N_obs = int(T / dt)
        T = N_obs * dt
        kwargs["T"] = T
        kwargs["dt"] = dt
        self.df = df = 1 / T
        f = np.arange(0.0, fmax + df, df)
        num = len(f)
        A_out = np.zeros(num, dtype=np.complex128)
        E_out = np.zeros(num, dtype=np.complex128)
        self.run_wave(*args, **kwargs)
        start = int(self.start_inds[0].item())
        A_temp = self.A_out.squeeze().cpu().numpy()
        E_temp = self.E_out.squeeze().cpu().numpy()
        A_out[start:start + self.N] = A_temp
        E_out[start:start + self.N] = E_temp
        return A_out, E_out

    # ---------------------------------------------------- information matrix
    def _transform_jacobian(self, params, parameter_transforms, step=1e-6):
        """D[b, k, l] = theta_l dphi_k/dtheta_l for phi = T(theta): the
        derivative of the transformed parameters along the reference's relative
        step theta (1 + eps e_l), by five-point differences of the transforms on
        the host (relative step 1e-6: truncation ~1e-24, rounding ~1e-11 of
        the transforms' scale).  A parameter of value 0 has a zero column, as
        the reference's relative step leaves it in place."""
        th = np.array(params, dtype=np.float64)
        n, B = th.shape
        D = np.zeros((B, n, n))

        def T(scale):
            return np.asarray(self._apply_parameter_transforms(th * scale, parameter_transforms),
                              dtype=np.float64)
        for l in range(n):
            sc = np.ones((n, 1))
            v = {}
            for k in (-2, -1, 1, 2):
                sc[l, 0] = 1.0 + k * step
                v[k] = T(sc)
            with np.errstate(invalid="ignore"):
                D[:, :, l] = ((8.0 * (v[1] - v[-1]) - (v[2] - v[-2])) / (12.0 * step)).T
        return D

    def _apply_parameter_transforms(self, params, parameter_transforms):
        for ind_trans, trans in parameter_transforms.items():
            if isinstance(ind_trans, int):
                params[ind_trans] = trans(params[ind_trans])
            else:
                params[np.asarray(ind_trans)] = trans(*params[np.asarray(ind_trans)])
        return params

    def information_matrix(self, params, eps=1e-9, parameter_transforms={}, inds=None, N=1024,
                           psd_func=None, psd_kwargs={}, easy_central_difference=False,
                           return_gpu=False, method="auto", **kwargs):
        """Fisher matrices of the reference's information_matrix (gbgpu.py:957-1138).

        The reference differentiates with relative steps, h(T(theta (1 +- eps)))
        with T the parameter transforms, so its matrices are in the logarithms
        of the sampled parameters: F_ij = <theta_i dh/dtheta_i | theta_j
        dh/dtheta_j>.  ``method="forward"`` forms them from the forward-mode
        kernel (``gbx_fisher``: one launch, exact derivatives in the physical
        parameters phi = T(theta); the 9-parameter model, equal arms, N <= 1024)
        by the chain rule, F = D^T F_phi D with D_kl = theta_l dphi_k/dtheta_l
        (``_transform_jacobian``; D = diag(theta) without transforms);
        ``"differences"`` runs the reference's central differences of run_wave;
        ``"auto"`` takes the first where it applies.
        """
        if psd_func is None:
            from .sensitivity import A1TDISens
            psd_func = A1TDISens.get_Sn
        if N is None:
            raise ValueError("N must be provided up front for Infromation Matrix.")
        if method not in ("auto", "forward", "differences"):
            raise ValueError("method must be 'auto', 'forward' or 'differences'")
        params = np.atleast_2d(_to_host(params))
        num_params = len(params)
        num_bins = len(params[0])
        if inds is None:
            inds = np.arange(num_params)
        fwd_ok = (num_params == 9 and not self.unequal_arms and
                  np.ndim(N) == 0 and int(N) <= 1024 and
                  set(kwargs) <= {"T", "dt", "tdi2", "oversample"})
        D = None
        if fwd_ok and method != "differences" and parameter_transforms:
            D = self._transform_jacobian(params, parameter_transforms)
            if not np.all(np.isfinite(D)):
                fwd_ok = False      # a transform left its domain within the stencil
        if method == "forward" and not fwd_ok:
            raise ValueError("forward-mode information matrices cover the 9-parameter model "
                             "with equal arms and N <= 1024, and parameter transforms "
                             "that are finite around the parameters")
        if method == "forward" or (method == "auto" and fwd_ok):
            T = kwargs.get("T", 4 * YRSID_SI)
            dt = kwargs.get("dt", 10.0)
            Tu = int(T / dt) * dt
            phys = np.array(params, dtype=np.float64)
            if parameter_transforms:
                phys = np.asarray(self._apply_parameter_transforms(phys, parameter_transforms),
                                  dtype=np.float64)
            prm = torch.as_tensor(np.ascontiguousarray(phys), device=self.device)
            F = self._fisher_forward(prm, int(N), Tu, Tu, bool(kwargs.get("tdi2", False)),
                                     psd_func, psd_kwargs)
            if D is None:
                th = torch.as_tensor(np.ascontiguousarray(params, dtype=np.float64).T,
                                     device=self.device)
                F = F * th[:, :, None] * th[:, None, :]      # d/d ln theta, as the reference
            else:
                Dd = torch.as_tensor(D, device=self.device)
                F = torch.einsum("bki,bkl,blj->bij", Dd, F, Dd)
            ix = torch.as_tensor(np.asarray(inds, dtype=np.int64), device=self.device)
            F = F[:, ix][:, :, ix].contiguous()
            return F if return_gpu else F.cpu().numpy()
        kwargs["N"] = N
        num_derivs = len(inds)
        info = torch.zeros((num_bins, num_derivs, num_derivs), dtype=torch.float64,
                           device=self.device)
        dh = torch.zeros((num_bins, num_derivs, 2, N), dtype=torch.complex128, device=self.device)

        def wave(step):
            p = self._apply_parameter_transforms(step * params, parameter_transforms)
            self.run_wave(*p, **kwargs)
            return torch.stack([self.A, self.E], 1)

        for i, ind in enumerate(inds):
            up1 = np.ones_like(params)
            up1[ind] += eps
            dn1 = np.ones_like(params)
            dn1[ind] -= eps
            h_up = wave(up1)
            h_dn = wave(dn1)
            if easy_central_difference:
                dh[:, i] = (h_up - h_dn) / (2 * eps)
            else:
                up2 = np.ones_like(params)
                up2[ind] += 2 * eps
                h_up2 = wave(up2)
                if not bool(torch.all(self.start_inds == self.start_inds[0])):
                    raise ValueError(
                        "The user should decrease steps size (eps) because the frequency bins "
                        "are changing during derivative calculation, which is not allowed.")
                dn2 = np.ones_like(params)
                dn2[ind] -= 2 * eps
                h_dn2 = wave(dn2)
                dh[:, i] = (-h_up2 + h_dn2 + 8 * (h_up - h_dn)) / (12 * eps)
        freqs = self.freqs
        psd = torch.as_tensor(np.asarray(psd_func(_to_host(freqs), **psd_kwargs)),
                              device=self.device)
        for i in range(num_derivs):
            for j in range(i, num_derivs):
                ip = 4 * self.df * torch.sum((dh[:, i].conj() * dh[:, j]).real / psd[:, None, :],
                                             dim=(1, 2))
                info[:, i, j] = ip
                info[:, j, i] = ip
        if not return_gpu:
            return info.cpu().numpy()
        return info

    def fisher_matrices(self, params, N, T=4 * YRSID_SI, dt=10.0, tdi2=False, inds=None,
                        psd_func=None, psd_kwargs={}, return_gpu=False, method="auto"):
        """Per-binary Fisher matrices F_ij = <dh/dtheta_i | dh/dtheta_j> (A and E)
        for a whole batch.

        ``method="forward"``: forward-mode derivatives in one launch
        (``gbx_fisher``: the bases of the two polarisations and five slow-part
        tangents transformed per binary, the 45 products summed per bin; mixed
        form, the 9-parameter model, equal arms, N <= 1024).
        ``method="differences"``: five-point FP64 central differences of the
        batched waveform in absolute parameter steps (any model, 4 waveform
        launches per parameter).  ``"auto"`` takes the first where it applies.

        Unlike ``information_matrix`` (the reference's, gbgpu.py:957-1138: steps
        relative to each parameter, and every binary of a call must share one
        start bin), binaries may sit anywhere: each derivative is taken on the
        binary's own window.  With differences the f0 stencil stays inside the
        binary's carrier bin rint(f0 T) (shortened near a bin edge), and a step
        that still moves the window is aligned before differencing.  ``params``
        is (nparams, B); ``inds`` selects the parameters (default all 9 / 14).
        Steps: amp 1e-6 amp; f0 1e-4/T; fdot 1e-4/T^2; fddot 1e-4/T^3
        (phase-equivalent); angles 1e-6 rad; third body: A2, P2 relative 1e-6,
        varpi, e2, T2 1e-6.  Returns (B, n, n) NumPy (or a CUDA tensor with
        ``return_gpu``).
        """
        if psd_func is None:
            from .sensitivity import A1TDISens
            psd_func = A1TDISens.get_Sn
        prm = _to_device(params, torch.float64, self.device).contiguous()
        npar, B = prm.shape
        if npar != self.NPARAMS:
            raise ValueError(f"params must be ({self.NPARAMS}, B)")
        inds = list(range(npar)) if inds is None else [int(i) for i in inds]
        Tu = int(T / dt) * dt
        N = int(N)
        if method not in ("auto", "forward", "differences"):
            raise ValueError("method must be 'auto', 'forward' or 'differences'")
        fwd_ok = npar == 9 and not self.unequal_arms and N <= 1024
        if method == "forward" and not fwd_ok:
            raise ValueError("forward-mode Fisher matrices cover the 9-parameter model, equal "
                             "arms and N <= 1024")
        if method == "forward" or (method == "auto" and fwd_ok):
            F = self._fisher_forward(prm, N, T, Tu, tdi2, psd_func, psd_kwargs)
            ix = torch.as_tensor(inds, device=self.device)
            F = F[:, ix][:, :, ix].contiguous()
            return F if return_gpu else F.cpu().numpy()
        absolute = {1: 1e-4 / Tu, 2: 1e-4 / Tu ** 2, 3: 1e-4 / Tu ** 3, 4: 1e-6, 5: 1e-6,
                    6: 1e-6, 7: 1e-6, 8: 1e-6, 10: 1e-6, 11: 1e-6, 13: 1e-6}

        def wave(p):
            self.run_wave(*p, N=N, T=T, dt=dt, tdi2=tdi2)
            return torch.stack([self.A, self.E], 1), self.start_inds.clone()

        h0, s0 = wave(prm)
        n = len(inds)
        dh = torch.zeros((B, n, 2, N), dtype=torch.complex128, device=self.device)
        cols = torch.arange(N, device=self.device)

        def aligned(h, s):
            # the window starting at bin s on the grid of the centre window s0:
            # out[i] = h[i - (s - s0)] where that index exists, else 0
            src = cols[None, :] - (s - s0)[:, None]
            ok = (src >= 0) & (src < N)
            idx = src.clamp(0, N - 1)[:, None, :].expand(-1, 2, -1)
            return torch.where(ok[:, None, :], torch.gather(h, 2, idx), torch.zeros_like(h))

        for i, ind in enumerate(inds):
            step = prm[ind].abs() * 1e-6 if ind in (0, 9, 12) else \
                torch.full((B,), absolute[ind], dtype=torch.float64, device=self.device)
            if ind == 1:
                # keep the stencil inside the carrier bin rint(f0 T): the
                # heterodyned model is not exactly invariant under a change of q
                frac = prm[1] * Tu - torch.round(prm[1] * Tu)
                room = (0.5 - frac.abs()) / Tu
                step = torch.minimum(step, torch.clamp(room / 2.5, min=1e-7 / Tu))
            step = torch.where(step > 0, step, torch.full_like(step, 1e-12))
            hs = []
            for m in (2, 1, -1, -2):
                q = prm.clone()
                q[ind] = q[ind] + m * step
                h, si = wave(q)
                hs.append(aligned(h, si))
            dh[:, i] = (-hs[0] + 8 * hs[1] - 8 * hs[2] + hs[3]) / (12 * step)[:, None, None]
        # the PSD on the union of the windows' bins (one host evaluation per
        # distinct bin), gathered per binary on the device
        lo = int(s0.min().item())
        hi = int(s0.max().item()) + N
        grid = np.asarray(psd_func((lo + np.arange(hi - lo)) / Tu, **psd_kwargs), dtype=np.float64)
        grid = torch.as_tensor(grid, device=self.device)
        psd = grid[(s0 - lo)[:, None] + cols[None, :]]             # (B, N)
        w = 4.0 / Tu / psd
        F = torch.einsum("bicn,bjcn->bij", dh.conj() * w[:, None, None, :], dh).real
        F = 0.5 * (F + F.transpose(1, 2))
        return F if return_gpu else F.cpu().numpy()

    def _fisher_forward(self, prm, N, T, Tu, tdi2, psd_func, psd_kwargs):
        """(B, 9, 9) Fisher matrices from gbx_fisher on the PSD of the union
        of the binaries' windows (one host evaluation per distinct bin)."""
        B = prm.shape[1]
        F = torch.zeros((B, 9, 9), dtype=torch.float64, device=self.device)
        if B == 0:
            return F
        self._check_T(Tu)
        q = torch.round(prm[1] * Tu).to(torch.int64) - N // 2
        lo = int(q.min().item()) - N
        hi = int(q.max().item()) + 2 * N
        grid = np.asarray(psd_func((lo + np.arange(hi - lo)) / Tu, **psd_kwargs), dtype=np.float64)
        psd = torch.as_tensor(grid, device=self.device).contiguous()
        plan = self._plan(N, Tu, "mixed", tdi2, 9)
        self._status.zero_()
        a = plan.args(prm, lo, self._status, grad=True)
        rc = nat.lib().gbx_fisher(ctypes.byref(a), psd.data_ptr(), psd.data_ptr(), int(hi - lo), 1,
                                  None, 1.0 / Tu, nat.ptr(F), nat.stream_handle())
        nat.check(rc, "gbx_fisher")
        self._check_status()
        return F

    # ----------------------------------------------------------------- hooks
    @abc.abstractmethod
    def add_to_argS(self, argS, f0, fdot, fddot, xi, *args):
        """Abstract hook: add a model's phase term to argS (gbgpu.py:1141-1168)."""
        raise NotImplementedError

    @abc.abstractmethod
    def prepare_additional_args(self, *args):
        """Abstract hook: convert a model's extra parameters (gbgpu.py:1170-1186)."""
        raise NotImplementedError

    @abc.abstractmethod
    def special_get_N(self, amp, f0, T, *args, oversample=1):
        """Abstract hook: N for a model's extra parameters (gbgpu.py:1188-1212)."""
        raise NotImplementedError

    @abc.abstractmethod
    def shift_frequency(self, fi, xi, *args):
        """Abstract hook: a model's shift of the instantaneous frequency (gbgpu.py:1214-1238)."""
        raise NotImplementedError


class GBGPU(GBGPUBase):
    """Circular Galactic binaries (reference gbgpu/gbgpu.py:1233-1327)."""

    def prepare_additional_args(self, *args):
        """No extra parameters: extra arguments are an error (gbgpu.py:1240-1257)."""
        raise ValueError(
            "If providing more args than the base args, must be a class derived from GBGPUBase "
            "with an adjusted 'prepare_additional_args' method.")

    def special_get_N(self, amp, f0, T, *args, oversample=1):
        """get_N's band table and SNR bump (gbgpu.py:1259-1282)."""
        return get_N(amp, f0, T, oversample=oversample)

    def shift_frequency(self, fi, xi, *args):
        """No shift of the instantaneous frequency (gbgpu.py:1284-1299)."""
        return fi

    def add_to_argS(self, argS, f0, fdot, fddot, xi, *args):
        """No extra phase term (gbgpu.py:1301-1327)."""
        return argS
