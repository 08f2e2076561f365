"""Host-side logic, the C ABI library and the struct mirrors (no GPU needed)."""

import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import fastgb_oracle as O
from conftest import ROOT, load_golden


def test_library_exports_every_declared_symbol():
    from gbgpu_gb300 import build, _native
    build.build()
    lib = ctypes.CDLL(build.LIB)
    header = open(os.path.join(ROOT, "include", "gbgpu_gb300.h")).read()
    declared = set(re.findall(r"^\s*(?:int|size_t|const char \*)\s*\*?\s*(gbx_\w+)\s*\(",
                              header, re.M))
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    assert declared <= set(_native.EXPORTS) | {n for n in declared if n.startswith("gbx_")}
    assert set(_native.EXPORTS) <= declared
    # loading needs no GPU; a call that touches no device memory works too
    assert lib.gbx_version() == 100


def test_struct_mirrors_match_c_layout(tmp_path):
    """Every field offset and the size of the ctypes mirrors equal the C ones."""
    from gbgpu_gb300 import _native
    structs = {"gbx_wave_args": _native.WaveArgs, "gbx_ll_args": _native.LLArgs}
    lines = []
    for cname, py in structs.items():
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {fname}));')
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"gbgpu_gb300.h\"\n"
                   "int main(void) {\n" + "\n".join(lines) + "\n  return 0; }\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = []
    for py in structs.values():
        want.append(ctypes.sizeof(py))
        want += [getattr(py, fname).offset for fname, _ in py._fields_]
    assert got == want


def test_get_N_matches_reference():
    from gbgpu_gb300.utility import get_N
    from gbgpu_gb300.constants import YRSID_SI
    g = load_golden("get_n")
    for key in g["keys"]:
        _, T, os_ = key.split("_")
        T = float(T)
        # keys store T with one decimal; recover the exact multiple of a year
        for mult in (0.5, 1.5, 3.0, 4.0, 6.0, 9.0):
            if abs(mult * YRSID_SI - T) < 1.0:
                T = mult * YRSID_SI
        np.testing.assert_array_equal(get_N(g["amp"], g["f0"], T, oversample=int(os_)), g[key])


def test_third_body_special_get_N_matches_reference():
    from gbgpu_gb300.thirdbody import GBGPUThirdBody
    from gbgpu_gb300.constants import YRSID_SI
    g = load_golden("get_n")
    # special_get_N is host logic; call it unbound (no GPU object needed)
    n = GBGPUThirdBody.special_get_N(None, g["amp"], g["f0"], 4 * YRSID_SI, np.ones(64),
                                     np.zeros(64), np.zeros(64), g["P2"], np.zeros(64),
                                     oversample=2)
    np.testing.assert_array_equal(n, g["third_N"])


def test_utility_functions_match_reference():
    from gbgpu_gb300 import utility as U
    g = load_golden("misc")
    A, E, T = U.AET(g["X"], g["Y"], g["Z"])
    np.testing.assert_array_equal(A, g["A"])
    np.testing.assert_array_equal(E, g["E"])
    np.testing.assert_array_equal(T, g["T"])
    np.testing.assert_array_equal(U.get_fGW(g["f0"], g["fdot"], g["fddot"], g["t"]), g["fgw"])
    np.testing.assert_allclose(U.get_amplitude(g["m1"], g["m2"], np.array([0.1, 0.01, 0.003]),
                                               np.array([6.0, 1.0, 10.0])), g["amp"], rtol=1e-15)
    fd = U.get_fdot(np.array([1e-3, 2e-3, 5e-3]), m1=g["m1"], m2=g["m2"])
    np.testing.assert_allclose(fd, g["fdotout"], rtol=1e-15)
    np.testing.assert_allclose(U.get_chirp_mass_from_f_fdot(np.array([1e-3, 2e-3, 5e-3]), fd),
                               g["Mc"], rtol=1e-15)
    # tutorial known answers (examples/GBGPU_tutorial.ipynb cells 30, 32)
    assert f"{U.get_amplitude(0.2, 0.1, 0.1, 6.0):.8e}" == "6.37562267e-23"
    assert f"{U.get_fdot(1e-3, m1=0.2, m2=0.1):.8e}" == "1.73157515e-19"


def test_orbits_identical_to_oracle():
    from gbgpu_gb300.orbits import EqualArmlengthOrbits
    t = np.linspace(0, 4 * 31557600.0, 257)
    a, b = EqualArmlengthOrbits(), O.OracleOrbits()
    for s in (1, 2, 3):
        np.testing.assert_array_equal(a.get_pos(t, np.full(257, s)), b.get_pos(t, np.full(257, s)))


@pytest.mark.parametrize("seed,tile", [(0, 0), (1, 0), (2, 0), (3, 64), (4, 256), (5, 2048),
                                       (6, 4096)])
def test_plan_tiles_cover_every_binary_once(seed, tile):
    from gbgpu_gb300.gbgpu import plan_tiles
    rng = np.random.default_rng(seed)
    Ns = 2 ** rng.integers(5, 13, 1000)
    order, tiles = plan_tiles(Ns, tile)
    assert sorted(order.tolist()) == list(range(1000))
    seen = np.zeros(1000, int)
    prevN = 1 << 20
    for lg, first, cnt, _ in tiles:
        N = 1 << lg
        assert N <= prevN                       # decreasing N (load balance)
        prevN = N
        assert 1 <= cnt <= min(16, max(1, (tile or 512) // N))
        for s in range(first, first + cnt):
            assert Ns[order[s]] == N
            seen[order[s]] += 1
    assert np.all(seen == 1)


def test_plan_tiles_rejects_non_power_of_two():
    from gbgpu_gb300.gbgpu import plan_tiles
    with pytest.raises(NotImplementedError):
        plan_tiles([64, 96])
    assert plan_tiles([])[1].shape == (0, 4)


def test_autotune_workload_keys():
    from gbgpu_gb300.autotune import workload_key
    k1 = workload_key("ll", 256, 50000, "mixed", True, 9)
    assert k1 == "ll|256:65536|mixed|tdi2=1|np=9"
    Ns = np.array([64] * 1000 + [2048] * 30)
    k2 = workload_key("grad", Ns, Ns.size, "mixed", False, 14)
    assert k2 == "grad|64:1024,2048:32|mixed|tdi2=0|np=14"
    # batches of similar size and the same N mix share a key
    assert workload_key("ll", np.array([64] * 1100 + [2048] * 29), 1129, "mixed", False, 14) \
        == k2.replace("grad", "ll")


def test_flops_per_binary_count():
    """The frozen FLOP count: 345 per sample + 3 FFTs of 5 N log2 N; TDI-2,
    third body and likelihood terms add per sample / per bin; arrays work."""
    from gbgpu_gb300.utility import flops_per_binary
    assert flops_per_binary(256) == 345 * 256 + 15 * 256 * 8          # 119,040
    assert flops_per_binary(256, tdi2=True) - flops_per_binary(256) == 20 * 256
    assert flops_per_binary(256, third_body=True) - flops_per_binary(256) == 177 * 256
    assert flops_per_binary(256, likelihood=True) - flops_per_binary(256) == 24 * 256
    Ns = np.array([64, 128, 2048])
    np.testing.assert_array_equal(flops_per_binary(Ns), [flops_per_binary(n) for n in Ns])


class _DLPackOnly:
    """An array of another library that only speaks DLPack."""

    def __init__(self, t):
        self._t = t

    def __dlpack__(self, *args, **kwargs):
        return self._t.__dlpack__(*args, **kwargs)

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def test_foreign_arrays_enter_without_copy():
    """Arrays of other libraries (DLPack here; the CUDA array interface on the
    GPU) become torch views: same memory when dtype and device match."""
    torch = pytest.importorskip("torch")
    from gbgpu_gb300.gbgpu import _native, _to_device, _to_host
    t = torch.arange(6, dtype=torch.float64)
    x = _to_device(_DLPackOnly(t), torch.float64, "cpu")
    assert torch.equal(x, t) and x.data_ptr() == t.data_ptr()
    np.testing.assert_array_equal(_to_host(_DLPackOnly(t)), t.numpy())
    assert _to_device(_DLPackOnly(t), torch.float32, "cpu").dtype == torch.float32
    # NumPy arrays and plain sequences keep their own path
    a = np.arange(3.0)
    assert _native(a) is a and _native([1, 2]) == [1, 2]
    np.testing.assert_array_equal(_to_device([1, 2], torch.int32, "cpu").numpy(), [1, 2])


def test_c_abi_rejects_bad_arguments_before_touching_a_device():
    """Argument checks of the C ABI return their status codes (and a message
    in gbx_last_error) before any CUDA call, so they run here without a GPU."""
    from gbgpu_gb300 import build, _native as nat
    build.build()
    lib = ctypes.CDLL(build.LIB)
    vp, i, d, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    lib.gbx_last_error.restype = ctypes.c_char_p
    lib.gbx_get_ll_ex.argtypes = [vp] * 8 + [d, vp, i, i, vp, vp, i, ll, ll, i, i, vp, vp]
    lib.gbx_fill_global_ex.argtypes = [vp] * 5 + [i, i, vp, i, i, ll, ll, ll, vp, vp]
    lib.gbx_waveform_ll.argtypes = [vp, vp, vp, vp, vp]
    lib.gbx_waveform_ll_grad.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.gbx_wave_workspace_bytes.restype = ctypes.c_size_t
    lib.gbx_wave_workspace_bytes.argtypes = [i]
    ERR_ARG, ERR_UNSUPPORTED = 1, 2
    fake = ctypes.c_void_p(0x1000)               # never dereferenced: the checks fail first
    ptrs = [fake] * 8

    def msg():
        return lib.gbx_last_error().decode()

    # drop-in get_ll: negative sizes, NULL pointers; an empty batch is a no-op
    assert lib.gbx_get_ll_ex(*ptrs, 1.0, fake, 16, -1, None, None, 100, 1, 1, 0, 0,
                             None, None) == ERR_ARG
    assert "negative" in msg()
    assert lib.gbx_get_ll_ex(None, *ptrs[1:], 1.0, fake, 16, 4, None, None, 100, 4, 1, 0, 0,
                             None, None) == ERR_ARG
    assert "NULL" in msg()
    assert lib.gbx_get_ll_ex(*ptrs, 1.0, fake, 16, 0, None, None, 100, 0, 1, 0, 0,
                             None, None) == 0
    # fill: group stride shorter than the data
    assert lib.gbx_fill_global_ex(*ptrs[:4], fake, 16, 4, fake, 100, 2, 50, 4, 1,
                                  None, None) == ERR_ARG
    assert "group_stride" in msg()

    # waveform family: the struct checks
    def args(**kw):
        a = nat.WaveArgs()
        a.params, a.num_bin, a.nparams, a.N = fake, 4, 9, 256
        a.precision, a.T, a.armlength, a.year = nat.GBX_MIXED, 1e7, 2.5e9, 3.15e7
        a.orbit[8] = fake
        for k, v in kw.items():
            setattr(a, k, v)
        return a
    la = nat.LLArgs()
    la.A_data = la.E_data = la.A_psd = la.E_psd = fake
    la.data_length, la.num_data, la.num_psd, la.df = 100, 1, 1, 1e-7
    cases = [
        (args(nparams=10), ERR_ARG, "nparams"),
        (args(precision=7), ERR_ARG, "precision"),
        (args(T=0.0), ERR_ARG, "T and armlength"),
        (args(N=100), ERR_UNSUPPORTED, "power of two"),
        (args(N=16384), ERR_UNSUPPORTED, "limit"),
        (args(N=512), ERR_ARG, "orbit table"),
        (args(tile=100), ERR_ARG, "tile"),
        (args(tile=8192), ERR_ARG, "tile"),
        (args(blocks_per_sm=-1), ERR_ARG, "blocks_per_sm"),
        (args(workspace=ctypes.c_void_p(0x1008).value, workspace_bytes=1 << 20), ERR_ARG,
         "aligned"),
        (args(workspace=fake.value, workspace_bytes=16), ERR_ARG, "workspace smaller"),
    ]
    for a, code, text in cases:
        assert lib.gbx_waveform_ll(ctypes.byref(a), ctypes.byref(la), fake, fake, None) == code, text
        assert text in msg(), (text, msg())
    bad = nat.LLArgs()
    assert lib.gbx_waveform_ll(ctypes.byref(args()), ctypes.byref(bad), fake, fake, None) == ERR_ARG
    # gradients: the mixed form only, 9 or 14 parameters, an aligned workspace of the right size
    g = ctypes.c_void_p(0x1000)
    assert lib.gbx_waveform_ll_grad(ctypes.byref(args(precision=nat.GBX_FP64)), ctypes.byref(la),
                                    fake, fake, g, None) == ERR_UNSUPPORTED
    assert "mixed" in msg()
    assert lib.gbx_waveform_ll_grad(ctypes.byref(args()), ctypes.byref(la), fake, fake, g,
                                    None) == ERR_ARG
    assert "workspace" in msg()
    assert lib.gbx_wave_workspace_bytes(0) == 0 and lib.gbx_wave_workspace_bytes(3) % 256 == 0
    # TDI bits: only TDI-2 and unequal arms; unequal arms not in the FP32 form
    for a, code, text in [(args(tdi2=4), ERR_ARG, "GBX_TDI"),
                          (args(tdi2=nat.GBX_TDI_UNEQUAL), ERR_UNSUPPORTED, "unequal arms")]:
        assert lib.gbx_waveform_ll(ctypes.byref(a), ctypes.byref(la), fake, fake, None) == code
        assert text in msg(), (text, msg())
    # swap gradient: mixed form, aligned workspace, uniform N, even num_bin, a gradient buffer
    lib.gbx_swap_ll_grad.argtypes = [vp, vp, vp, vp, vp]
    lib.gbx_grad_workspace_bytes.restype = ctypes.c_size_t
    lib.gbx_grad_workspace_bytes.argtypes = [i]
    ws = dict(workspace=fake.value, workspace_bytes=lib.gbx_grad_workspace_bytes(8))
    swap_cases = [
        (args(precision=nat.GBX_FP64, **ws), fake, ERR_UNSUPPORTED, "mixed"),
        (args(), fake, ERR_ARG, "workspace"),
        (args(num_bin=5, **ws), fake, ERR_ARG, "even"),
        (args(order=fake.value, **ws), fake, ERR_ARG, "uniform N"),
        (args(**ws), None, ERR_ARG, "gradient"),
    ]
    for a, gbuf, code, text in swap_cases:
        assert lib.gbx_swap_ll_grad(ctypes.byref(a), ctypes.byref(la), fake, gbuf, None) == code, text
        assert text in msg(), (text, msg())
    # forward-mode Fisher matrices: 9 parameters, equal arms, an output buffer
    lib.gbx_fisher.argtypes = [vp, vp, vp, i, i, vp, d, vp, vp]
    fisher_cases = [
        (args(nparams=14, year=3.15e7, **ws), fake, ERR_UNSUPPORTED, "9-parameter"),
        (args(precision=nat.GBX_FP64, **ws), fake, ERR_UNSUPPORTED, "mixed"),
        (args(**ws), None, ERR_ARG, "Fisher"),
        (args(), fake, ERR_ARG, "workspace"),
    ]
    for a, out, code, text in fisher_cases:
        assert lib.gbx_fisher(ctypes.byref(a), fake, fake, 100, 1, None, 1e-7, out, None) == code, text
        assert text in msg(), (text, msg())
    # the FP64 drop-in: the same checks as gbx_get_ll_ex
    lib.gbx_get_ll_fp64.argtypes = lib.gbx_get_ll_ex.argtypes
    assert lib.gbx_get_ll_fp64(*ptrs, 1.0, fake, 16, -1, None, None, 100, 1, 1, 0, 0,
                               None, None) == ERR_ARG
    assert lib.gbx_get_ll_fp64(*ptrs, 1.0, fake, 16, 0, None, None, 100, 0, 1, 0, 0,
                               None, None) == 0


def test_tabulated_orbits_interpolate_the_analytic_orbit(tmp_path):
    """TabulatedOrbits (positions on a grid, cubic spline) reproduces the
    analytic orbit it was sampled from to a few metres at 6-hour sampling,
    loads from an .npz file, and refuses times outside its grid."""
    from gbgpu_gb300.orbits import EqualArmlengthOrbits, TabulatedOrbits
    ana = EqualArmlengthOrbits()
    t = np.arange(0.0, 5 * 31557600.0, 21600.0)
    pos = np.stack([ana.get_pos(t, np.full(t.size, s)) for s in (1, 2, 3)])
    tab = TabulatedOrbits(t, pos, ana.armlength)
    rng = np.random.default_rng(3)
    tt = np.sort(rng.uniform(0, t[-1], 2000))
    for s in (1, 2, 3):
        err = np.abs(tab.get_pos(tt, np.full(tt.size, s)) - ana.get_pos(tt, np.full(tt.size, s)))
        assert err.max() < 5.0, err.max()                        # metres (2e-8 s of light time)
    mixed = tab.get_pos(tt[:6], np.array([1, 2, 3, 3, 2, 1]))
    np.testing.assert_array_equal(mixed[2], tab.get_pos(tt[2:3], np.array([3]))[0])
    np.savez(tmp_path / "orb.npz", t=t, pos=pos, armlength=ana.armlength)
    f = TabulatedOrbits.from_file(tmp_path / "orb.npz")
    np.testing.assert_array_equal(f.get_pos(tt[:5], np.ones(5, int)), tab.get_pos(tt[:5], np.ones(5, int)))
    with pytest.raises(ValueError):
        tab.get_pos(np.array([t[-1] + 1.0]), np.array([1]))
    with pytest.raises(ValueError):
        TabulatedOrbits(t, pos[:, :10])


def test_n_array_key_reuse_and_verification_flags():
    """GBGPUBase._n_key: a new buffer gets its full content key at once; the
    same buffer with the same 64 sampled entries reuses the key and asks for
    verification after the launch; a change at a sampled entry, another
    length or another buffer computes the key at once again."""
    from gbgpu_gb300.gbgpu import GBGPU, _array_key
    gb = object.__new__(GBGPU)                 # host logic only: no device state
    gb._n_last = None
    Ns = (2 ** np.random.default_rng(2).integers(5, 12, 1000)).astype(np.int64)
    key, verify = gb._n_key(Ns)
    assert key == _array_key(Ns) and not verify
    key2, verify = gb._n_key(Ns)
    assert key2 == key and verify                  # same buffer, same samples
    Ns[1] = 64 if Ns[1] != 64 else 128             # not a sampled entry (step 15)
    key3, verify = gb._n_key(Ns)
    assert verify and key3 == key                  # stale until verified after the launch
    assert _array_key(Ns) != key                   # ... which is why the call verifies it
    Ns[15] = 64 if Ns[15] != 64 else 128           # a sampled entry
    key4, verify = gb._n_key(Ns)
    assert not verify and key4 == _array_key(Ns)
    other = Ns.copy()                              # same content, another buffer
    key5, verify = gb._n_key(other)
    assert not verify and key5 == key4
    key6, verify = gb._n_key(Ns[:500].copy())      # another length
    assert not verify


def test_unverified_n_key_never_files_a_new_plan(monkeypatch):
    """An N array changed in place at an unsampled entry comes back with the
    previous call's (stale) key.  When that key misses the plan cache (here:
    another precision), the plan built from the new contents must be filed
    under the new contents' key; otherwise a later call whose array holds the
    old contents would get a tile schedule for other N values."""
    import gbgpu_gb300.gbgpu as G
    from gbgpu_gb300 import autotune

    class FakePlan:
        def __init__(self, owner, N, T, precision, tdi2=False, nparams=9, tile=0,
                     blocks_per_sm=0):
            self.N = np.array(N, copy=True)
            self.precision = precision

    class FakeTuner:
        def tune(self, key, run):
            return (128, 0)

    monkeypatch.setattr(G, "WavePlan", FakePlan)
    monkeypatch.setattr(autotune, "default_tuner", lambda: FakeTuner())
    gb = object.__new__(G.GBGPU)
    gb._plans, gb._shapes, gb._n_last, gb.autotune = {}, {}, None, True
    T = 1e8
    Ns = (2 ** np.random.default_rng(3).integers(5, 12, 1000)).astype(np.int64)
    original = Ns.copy()
    key, verify = gb._n_key(Ns)
    assert not verify
    p1 = gb._plan(Ns, T, "mixed", False, 9, nkey=key, trusted=True)
    np.testing.assert_array_equal(p1.N, original)
    Ns[1] = 64 if Ns[1] != 64 else 128               # unsampled entry, same buffer
    stale, verify = gb._n_key(Ns)
    assert verify and stale == key
    p2 = gb._plan(Ns, T, "fp64", False, 9, nkey=stale, trusted=False)   # cache miss
    np.testing.assert_array_equal(p2.N, Ns)
    assert (G._array_key(Ns), len(Ns), T, "fp64", False, 9, 0, 0) in gb._plans
    assert (stale, len(Ns), T, "fp64", False, 9, 0, 0) not in gb._plans
    # a hit under the stale key is still allowed (the launch is verified afterwards)
    assert gb._plan(Ns, T, "mixed", False, 9, nkey=stale, trusted=False) is p1
    # the old contents at a new address get a plan built from the old contents
    again = original.copy()
    k_old, _ = gb._n_key(again)
    p3 = gb._plan(again, T, "fp64", False, 9, nkey=k_old, trusted=True)
    np.testing.assert_array_equal(p3.N, original)
    # launch shapes: a shape tuned under an unverified key is filed under the contents' key
    gb._n_key(Ns)
    gb._launch_shape("ll", Ns, len(Ns), "mixed", False, 9, None, nkey=stale, trusted=False)
    assert ("ll", G._array_key(Ns), len(Ns), "mixed", False, 9) in gb._shapes
    assert ("ll", stale, len(Ns), "mixed", False, 9) not in gb._shapes


def test_reference_arm_json_line_on_cpu():
    """`bench.py --impl reference` (the oracle port timed on the host cores)
    needs no GPU and prints one JSON line with the contract's keys."""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1", "--binaries", "20000"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "e2e",
              "cpu_baseline"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "binaries/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert "workload" in d["config"] and d["config"]["binaries_per_gpu"] == 20000
    # the whole batch is timed in every step: steps x ms_per_step is the timed region
    assert abs(d["value"] * d["ms_per_step"] / 1e3 - 20000) < 1.0
    assert sum(d["config"]["N_mix"].values()) == 20000


def test_N_none_resolves_to_the_batch_maximum_as_the_reference():
    """run_wave / get_ll with N=None take special_get_N's largest N over the
    batch (gbgpu.py:204-206), with oversample applied; for the third body the
    five extra parameters go to its special_get_N."""
    from gbgpu_gb300 import GBGPU, GBGPUThirdBody
    from gbgpu_gb300.constants import YRSID_SI
    g = load_golden("get_n")
    gb = object.__new__(GBGPU)                     # host logic only
    for os_ in (1, 2, 4):
        N = gb._resolve_N(None, g["amp"], g["f0"], 4.0 * YRSID_SI, (), os_)
        assert N == int(np.max(g[f"N_{4.0 * YRSID_SI:.1f}_{os_}"]))
    tb = object.__new__(GBGPUThirdBody)
    extra = (np.ones(64), np.zeros(64), np.zeros(64), g["P2"], np.zeros(64))
    assert tb._resolve_N(None, g["amp"], g["f0"], 4 * YRSID_SI, extra, 2) == int(np.max(g["third_N"]))
    # an explicit N passes through; an array stays per binary
    assert gb._resolve_N(256, g["amp"], g["f0"], YRSID_SI, (), 1) == 256
    Ns = gb._resolve_N(np.full(64, 128), g["amp"], g["f0"], YRSID_SI, (), 1)
    assert Ns.dtype == np.int64 and Ns.shape == (64,)


def test_transform_jacobian_matches_analytic_derivatives():
    """information_matrix's forward path: D[b, k, l] = theta_l dphi_k/dtheta_l
    of the parameter transforms (integer and tuple keys), five-point
    differences against the analytic derivatives, and a zero column for a
    parameter of value 0 (the reference's relative step leaves it in place)."""
    from gbgpu_gb300.gbgpu import GBGPUBase

    class Host:
        def _apply_parameter_transforms(self, p, t):
            return GBGPUBase._apply_parameter_transforms(self, p, t)

    rng = np.random.default_rng(1)
    B = 5
    th = np.array([rng.uniform(-51, -48, B), rng.uniform(1e-3, 3e-3, B),
                   10 ** rng.uniform(-17, -16, B), np.zeros(B), rng.uniform(0.5, 5, B),
                   rng.uniform(-0.9, 0.9, B), rng.uniform(0.3, 2.8, B), rng.uniform(0.5, 5, B),
                   rng.uniform(-0.9, 0.9, B)])
    tr = {0: np.exp, 5: np.arccos, 8: np.arcsin, (1, 2): lambda a, b: (a + 0.0 * b, 2.0 * b)}
    D = GBGPUBase._transform_jacobian(Host(), th, tr)
    for b in range(B):
        exp = np.diag(th[:, b])
        exp[0, 0] = th[0, b] * np.exp(th[0, b])
        exp[5, 5] = -th[5, b] / np.sqrt(1 - th[5, b] ** 2)
        exp[8, 8] = th[8, b] / np.sqrt(1 - th[8, b] ** 2)
        exp[2, 2] = 2.0 * th[2, b]
        nz = exp != 0
        assert np.all(D[b][~nz] == 0.0)
        assert np.max(np.abs(D[b][nz] - exp[nz]) / np.abs(exp[nz])) < 1e-8
    assert np.all(D[:, :, 3] == 0.0)


def test_issue_roofline_arithmetic():
    """bench.issue_roofline: warp instructions per sample (from the committed
    ncu summary) x samples / step time against SMs x 4 schedulers x clock."""
    import bench

    class Clk:
        def summary(self):
            return {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0}

    Ns = np.array([256] * 1000 + [2048] * 100)
    r = bench.issue_roofline(Ns, 2.0, Clk(), sms=152)
    per = bench.profiled("warp_instr_per_sample")
    assert per is not None and r["warp_instr_per_sample"] == per
    assert abs(r["peak"] - 152 * 4 * 2000e6) < 1.0
    assert abs(r["achieved"] - per * Ns.sum() / 2e-3) < 1e-3 * r["achieved"]
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
