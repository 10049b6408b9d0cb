"""red_calc_accel_noalloc: gravity without device allocation.

Callers whose GPU memory is owned by another pool, or that must not enter the
allocator, get gravity (and drag) from buffers they own; the library's
temporaries sit in a fixed __device__ array.  This file is collected last so
that a failure here leaves every other test already run; it passes alone in
a fresh process and after the other tests.

The entry point is checked through the C ABI against the allocating entry
point (red_calc_dydx with i = 1) on two calls in a row with different
systems, so that nothing left in the shared array by the first call leaks
into the second.  Tolerance: the same launch plan and summation order (the
allocating side keeps the global chunk reduction, REDGB_CLUSTER=0, as the
allocation-free entry point does), so the results agree to 1e-12 relative
(they are expected to be identical).  At the largest accepted size, a dense
system whose chunked plan would overflow the scratch array, the entry point
sums each sink's sources in one CTA instead of in chunks.  That regroups the
pair terms into other FP32 tile partials before their double-single sum, so
the plans agree to MIXED's stated tolerances there: 2e-6 for the star, whose
acceleration is a sum of FP32 pair terms only (the disk's pulls on it
largely cancel), and 1e-8 for the other bodies (the all-pairs bound of the
gravity parity tests; their double-single star term dominates).

A live simulation must not notice the entry point: a Sim stepped across a
call follows the same trajectory, bit for bit, as one that never saw it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def vec(a):
    return np.stack([a["x"], a["y"], a["z"]], axis=1)


def device_args(rg, torch, s, precision, t=0.0, gas=None):
    dev = torch.device("cuda:0")
    keep = {
        "r": torch.from_numpy(np.ascontiguousarray(vec(s.r)).reshape(-1)).to(dev),
        "v": torch.from_numpy(np.ascontiguousarray(vec(s.v)).reshape(-1)).to(dev),
        "mass": torch.from_numpy(np.ascontiguousarray(s.p["mass"])).to(dev),
        "radius": torch.from_numpy(np.ascontiguousarray(s.p["radius"])).to(dev),
        "density": torch.from_numpy(np.ascontiguousarray(s.p["density"])).to(dev),
        "cd": torch.from_numpy(np.ascontiguousarray(s.p["cd"])).to(dev),
        "id": torch.from_numpy(np.ascontiguousarray(s.md["id"]).astype(np.int32)).to(dev),
        "accel": torch.full((3 * s.n,), float("nan"), dtype=torch.float64, device=dev),
    }
    from redgb.lib import AccelArgs, PRECISION, gas_struct
    a = AccelArgs()
    for k in range(7):
        a.playing[k] = int(s.playing[k])
    for f in ("r", "v", "mass", "radius", "density", "cd", "id", "accel"):
        setattr(a, f, keep[f].data_ptr())
    a.precision = PRECISION[precision]
    a.t = t
    if gas is not None:
        a.gas_disk = 1
        a.gas = gas_struct(gas)
    a.device = 0
    a.stream = torch.cuda.current_stream().cuda_stream
    return a, keep


def reference(rg, s, precision, t=0.0, gas=None):
    import os
    old = os.environ.get("REDGB_CLUSTER")
    os.environ["REDGB_CLUSTER"] = "0"
    try:
        with rg.Sim(s, dt=0.01, precision=precision, gas=gas) as sim:
            return vec(sim.calc_dydx(0, 1, t))
    finally:
        if old is None:
            del os.environ["REDGB_CLUSTER"]
        else:
            os.environ["REDGB_CLUSTER"] = old


@pytest.mark.parametrize("precision", ["mixed", "fp32", "fp64", "fp64_exact"])
def test_noalloc_matches_allocating_entry_point_twice(rg, precision):
    torch = pytest.importorskip("torch")
    from redgb.lib import calc_accel_noalloc
    systems = [rg.ic.config1(seed=41, n_pl=2048), rg.ic.config2(seed=42, n_pp=8, n_pl=3000)]
    for s in systems:                               # two calls in a row, different systems
        ref = reference(rg, s, precision)
        a, keep = device_args(rg, torch, s, precision)
        calc_accel_noalloc(a)
        torch.cuda.synchronize()
        got = keep["accel"].cpu().numpy().reshape(-1, 3)
        assert np.all(np.isfinite(got))
        err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert err.max() <= 1e-12, err.max()


def test_noalloc_drag_matches(rg):
    torch = pytest.importorskip("torch")
    from redgb.lib import calc_accel_noalloc
    s = rg.ic.config3(n_pp=3, n_pl=500, seed=6)
    gas = np.array([rg.ic.gas_params(rg.ic.gas_disk_config3())], dtype=rg.types.GAS)[0]
    t = 3.0 * rg.ic.K
    ref = reference(rg, s, "mixed", t=t, gas=gas)
    a, keep = device_args(rg, torch, s, "mixed", t=t, gas=gas)
    calc_accel_noalloc(a)
    torch.cuda.synchronize()
    got = keep["accel"].cpu().numpy().reshape(-1, 3)
    err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() <= 1e-12


def test_noalloc_rejects_oversized_systems(rg):
    from redgb.lib import AccelArgs, NOALLOC_MAX_BODIES, RedError, calc_accel_noalloc
    a = AccelArgs()
    a.playing[5] = NOALLOC_MAX_BODIES + 1
    a.r = a.mass = a.id = a.accel = 16      # never dereferenced: the size check comes first
    with pytest.raises(RedError) as e:
        calc_accel_noalloc(a)
    assert e.value.code == 1 and "RED_NOALLOC_MAX_BODIES" in str(e.value)


def test_noalloc_leaves_live_simulations_alone(rg):
    """Steps of a Sim created before a call match those of a Sim that never saw one."""
    torch = pytest.importorskip("torch")
    from redgb.lib import calc_accel_noalloc
    s = rg.ic.config2(seed=43, n_pp=6, n_pl=1500)
    other = rg.ic.config1(seed=44, n_pl=700)
    runs = []
    for with_call in (False, True):
        with rg.Sim(s, dt=0.5 * rg.ic.K, precision="mixed") as sim:
            for k in range(6):
                if with_call and k in (1, 4):
                    a, keep = device_args(rg, torch, other, "fp64")
                    calc_accel_noalloc(a)
                    torch.cuda.synchronize()
                sim.step()
            st = sim.get_state(0)
            runs.append((vec(st.r), vec(st.v), sim.info(0).t))
    assert runs[0][2] == runs[1][2]
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def test_noalloc_largest_dense_system(rg):
    """RED_NOALLOC_MAX_BODIES bodies, every pair interacting (all protoplanets)."""
    torch = pytest.importorskip("torch")
    from redgb.lib import NOALLOC_MAX_BODIES, calc_accel_noalloc
    s = rg.ic.config2(seed=45, n_pp=16, n_pl=NOALLOC_MAX_BODIES - 17).relabel_all_SI()
    assert s.n == NOALLOC_MAX_BODIES
    ref = reference(rg, s, "mixed")
    for _ in range(2):
        a, keep = device_args(rg, torch, s, "mixed")
        calc_accel_noalloc(a)
        torch.cuda.synchronize()
        got = keep["accel"].cpu().numpy().reshape(-1, 3)
        err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert err[0] <= 2e-6, err[0]
        assert err[1:].max() <= 1e-8, err[1:].max()


def test_noalloc_restores_current_device(rg):
    torch = pytest.importorskip("torch")
    from redgb.lib import calc_accel_noalloc
    s = rg.ic.config1(seed=46, n_pl=300)
    before = torch.cuda.current_device()
    a, keep = device_args(rg, torch, s, "mixed")
    calc_accel_noalloc(a)
    torch.cuda.synchronize()
    assert torch.cuda.current_device() == before
