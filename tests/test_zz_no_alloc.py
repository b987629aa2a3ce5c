"""The allocation-free material-point entry point, checked against the allocating one.

nf_material_point_update_static exists for callers that cannot allocate device memory (the
allocating entry point's cudaMalloc/cudaFree synchronise the whole device, and a process whose
GPU memory belongs to its own pool allocator has none to spare). It stages through a fixed
device array instead. This test calls both entry points through the C ABI on the same inputs,
twice in a row (the second call starting from the first call's results, so the shared array is
reused with different contents), and requires bit-identical outputs -- the tolerance of every
other parity test in this suite -- also at exactly the array's capacity with damage on (the
top of the array in use). It checks that a request above the capacity is refused, and that a
call neither waits for nor holds up work the caller has queued on another stream. This file
sorts last so that a run stopping at the first failure has run everything else first.
"""
import ctypes as C
import time

import numpy as np
import pytest

from neofiz_gb300 import JohnsonCook, Material, _abi
from neofiz_gb300.solver import _dptr

pytestmark = pytest.mark.gpu

CAPACITY = 8192


def _bind(lib):
    fn = lib.nf_material_point_update_static
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(_abi.MaterialC), C.c_int32, C.c_int32, _abi.c_double_p,
                   _abi.c_double_p, _abi.c_double_p, _abi.c_double_p, _abi.c_double_p,
                   C.c_double, C.POINTER(_abi.DamagePoints), _abi.c_double_p]
    return fn


def _damage_struct(d):
    s = _abi.DamagePoints()
    for k in ("failure_strain", "fracture_energy", "youngs_modulus", "geometry", "strength",
              "softening", "width"):
        setattr(s, k, _dptr(d[k]))
    return s


def _call(fn, material, state, strain, damage):
    sig, back, eps, work = state
    dg = np.zeros(eps.size)
    ds = _damage_struct(damage) if damage is not None else None
    st = fn(C.byref(_abi.material_struct(material)), 1, eps.size, _dptr(sig), _dptr(back),
            _dptr(eps), _dptr(work), _dptr(strain), 1.0e-8,
            C.byref(ds) if ds is not None else None, _dptr(dg))
    assert st == 0
    return dg


@pytest.mark.parametrize("kind,n", [("linear", 6000), ("jc-damage", 6000),
                                    ("jc-damage", CAPACITY)])
def test_static_entry_matches_allocating_entry(gpu_lib, kind, n):
    lib = gpu_lib.lib
    static = _bind(lib)
    allocating = gpu_lib.material_point_update
    rng = np.random.default_rng((7 if kind == "linear" else 11) + n)
    if kind == "linear":
        m = Material.STEEL_4340.yielding(800e6, 1e9, 2e9)
    else:
        m = Material.COPPER_OFHC.withKinematicHardening(1e8).withJohnsonCook(
            JohnsonCook.COPPER_OFHC)
    sig = rng.normal(0.0, 3e8, 4 * n)
    back = rng.normal(0.0, 5e7, 4 * n)
    eps = np.abs(rng.normal(0.0, 0.2, n))
    work = np.abs(rng.normal(0.0, 2e8, n))
    a = [sig.copy(), back.copy(), eps.copy(), work.copy()]
    b = [sig.copy(), back.copy(), eps.copy(), work.copy()]
    dmg_a = dmg_b = None
    if kind == "jc-damage":
        dmg_a = {"failure_strain": np.abs(rng.normal(0.3, 0.1, n)) + 0.01,
                 "fracture_energy": np.full(n, 2e4), "youngs_modulus": np.full(n, m.youngsModulus),
                 "geometry": np.tile([1e-6, 1e-3, 1e-4, -2e-4, 1e-3], n).astype(np.float64),
                 "strength": np.zeros(n), "softening": np.zeros(n), "width": np.zeros(n)}
        dmg_b = {k: v.copy() for k, v in dmg_a.items()}
    for call in range(2):
        strain = rng.normal(0.0, 2e-3, 4 * n)
        dg_a = _call(static, m, a, strain, dmg_a)
        dg_b = np.zeros(n)
        ds = _damage_struct(dmg_b) if dmg_b is not None else None
        st = allocating(C.byref(_abi.material_struct(m)), 1, n, _dptr(b[0]), _dptr(b[1]),
                        _dptr(b[2]), _dptr(b[3]), _dptr(strain), 1.0e-8,
                        C.byref(ds) if ds is not None else None, _dptr(dg_b))
        assert st == 0
        assert np.array_equal(dg_a.view(np.uint64), dg_b.view(np.uint64)), f"call {call}"
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), f"call {call}"
        if dmg_a is not None:
            for k in ("strength", "softening", "width"):
                assert np.array_equal(dmg_a[k].view(np.uint64), dmg_b[k].view(np.uint64))
    assert np.count_nonzero(dg_a) > 0


def test_static_entry_refuses_more_than_its_capacity(gpu_lib):
    lib = gpu_lib.lib
    static = _bind(lib)
    n = CAPACITY + 1
    z4, z1 = np.zeros(4 * n), np.zeros(n)
    st = static(C.byref(_abi.material_struct(Material.STEEL_4340)), 1, n, _dptr(z4),
                _dptr(z4.copy()), _dptr(z1), _dptr(z1.copy()), _dptr(z4.copy()), 1e-8, None,
                _dptr(z1.copy()))
    assert st == _abi.NF_EINVAL
    assert str(CAPACITY) in gpu_lib.last_error(None).decode()


def test_static_entry_does_not_wait_for_the_callers_other_streams(gpu_lib):
    """The caller keeps the legacy default stream (a blocking stream, which every blocking
    stream waits for) busy with a bounded sleep of about a second; the call runs on the
    library's own non-blocking stream and returns while that sleep is still running."""
    torch = pytest.importorskip("torch")
    static = _bind(gpu_lib.lib)
    m = Material.STEEL_4340.yielding(800e6, 1e9, 2e9)
    n = 256
    rng = np.random.default_rng(3)
    state = [rng.normal(0.0, 3e8, 4 * n), rng.normal(0.0, 5e7, 4 * n),
             np.abs(rng.normal(0.0, 0.2, n)), np.abs(rng.normal(0.0, 2e8, n))]
    strain = rng.normal(0.0, 2e-3, 4 * n)
    _call(static, m, state, strain, None)            # the device's first call: set-up
    torch.cuda.synchronize()
    legacy = torch.cuda.default_stream()
    with torch.cuda.stream(legacy):
        torch.cuda._sleep(2_000_000_000)             # ~1 s of GPU clock cycles, bounded
    t0 = time.perf_counter()
    _call(static, m, state, strain, None)
    elapsed = time.perf_counter() - t0
    still_busy = not legacy.query()
    torch.cuda.synchronize()
    assert still_busy and elapsed < 0.5, f"the call waited {elapsed:.3f} s for another stream"
