"""Pins against red's own GPU path, built from its unmodified sources.

red's CPU path throws on planetesimals (src/red.cuda/pp_disk.cu:974-982), so
the oracle's GPU semantics -- the SI / NSI / NI interaction bounds of
calc_grav_accel_naive (pp_disk.cu:373-416, red_type.h:670-692) and the
collision loop that takes the star as i (pp_disk.cu:320-371) -- are a
restatement.  These tests run red's own kernels (oracle/ref_gpu.py drives
oracle/ref_harness.cu with dev=gpu) on the workloads' inputs at full size and
compare three things on the same inputs: red's GPU result, the oracle's
restatement and this library's FP64_EXACT mode.

Tolerances:
  * gravity (no drag), collision pairs and distances, fixed-step
    trajectories: bit-identical (red is built with -fmad=false, the oracle
    with -ffp-contract=off, FP64_EXACT uses red's operation order without
    FMA; sqrt and division are correctly rounded on both sides).
  * gravity with gas drag: 1e-14 relative to the acceleration.  The drag uses
    pow and exp, whose CUDA and glibc results may differ in the last bit.
  * adaptive RKF7(8): red's GPU run and the oracle take the same step sizes
    bit for bit (both form the step-size factor with the C library's pow on
    the host).  This library forms it on the device with the nearest double
    of the power (crmath.cuh), which the C library's pow returns except in
    rare misrounded cases (about 1 in 1000 calls): step counters equal, t to
    1e-8 and positions to 1e-7 relative (the embedded error estimate magnifies
    a 1-ulp difference of one step-size factor), and bit-identical when no
    call differed.

The staged sources (baseline/_ref, oracle/ref_stage.sh) are git-ignored; the
tests skip when they are absent.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NTHREADS = 16


def vec(a):
    return np.stack([a["x"], a["y"], a["z"]], axis=1)


@pytest.fixture(scope="module")
def red_gpu():
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("red's sources are not staged under baseline/_ref")
    ref_gpu.build()
    return ref_gpu


def obody(orc, s):
    return orc.Body(s.r, s.v, s.p, s.md, s.playing)


def test_red_gpu_gravity_disk16384_bitexact(rg, orc, red_gpu):
    """The 16384-body disk: 17 SI sinks against all, 16367 NSI sinks against the SI bodies."""
    s = rg.ic.config2()
    a_red = vec(red_gpu.accel(rg, s))
    _, a_orc = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU, nthreads=NTHREADS)
    assert np.array_equal(a_red, vec(a_orc))
    with rg.Sim(s, dt=0.01, precision="fp64_exact", stage_exact=True) as sim:
        a_lib = vec(sim.calc_dydx(0, 1, 0.0))
    assert np.array_equal(a_red, a_lib)


def test_red_gpu_gravity_test_particles_and_inactive(rg, orc, red_gpu):
    """NI sinks (test particles) and inactive bodies (id < 0) in every class."""
    rng = np.random.Generator(np.random.MT19937(17))
    s = rg.ic.build_system(rng, pp_a=np.array([0.8, 1.0, 1.2, 1.4]), pp_mass=0.1 * rg.ic.EARTH_TO_SOLAR,
                           pl_a=rng.uniform(0.7, 1.5, 3000), pl_mass=rg.ic.EARTH_TO_SOLAR / 3000, n_tp=500)
    for k in (2, 9, 700, s.n - 3):
        s.md["id"][k] *= -1
    a_red = vec(red_gpu.accel(rg, s))
    _, a_orc = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU, nthreads=NTHREADS)
    assert np.array_equal(a_red, vec(a_orc))
    with rg.Sim(s, dt=0.01, precision="fp64_exact", stage_exact=True) as sim:
        a_lib = vec(sim.calc_dydx(0, 1, 0.0))
    act = s.md["id"] > 0
    assert np.array_equal(a_red[act], a_lib[act])


def test_red_gpu_gravity_and_drag_disk65536(rg, orc, red_gpu):
    """The gas-drag disk (32 protoplanets, 65503 planetesimals) at t = 1.25 yr."""
    s = rg.ic.config3()
    keys = rg.ic.gas_disk_config3()
    gas = np.array([rg.ic.gas_params(keys)], dtype=rg.types.GAS)
    t = 1.25 * 365.25 * rg.ic.K
    a_red = vec(red_gpu.accel(rg, s, t=t, gas_keys=keys))
    _, a_orc = orc.calc_dydx(obody(orc, s), 1, t, gas=np.ascontiguousarray(gas, dtype=orc.GAS),
                             sem=orc.SEM_GPU, nthreads=NTHREADS)
    a_orc = vec(a_orc)
    scale = np.linalg.norm(a_orc, axis=1)
    assert (np.linalg.norm(a_red - a_orc, axis=1) / scale).max() <= 1e-14
    with rg.Sim(s, dt=0.01, precision="fp64_exact", stage_exact=True, gas=gas[0]) as sim:
        a_lib = vec(sim.calc_dydx(0, 1, t))
    assert (np.linalg.norm(a_red - a_lib, axis=1) / scale).max() <= 1e-14
    _, grav = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU, nthreads=NTHREADS)
    assert np.abs(a_red - vec(grav)).max() > 0.0     # the drag acts


def test_red_gpu_rk4_disk2053_bitexact(rg, orc, red_gpu):
    """The 2053-body disk at its full length: fixed-step RK4, dt = 0.5 d, 2000 steps (1000 d)."""
    s = rg.ic.config1()
    dt = 0.5 * rg.ic.K
    n = 2000
    red = red_gpu.run(rg, s, "rk4", dt, n)
    b = obody(orc, s)
    ig = orc.make_integrator(orc.RK4, dt, sem=orc.SEM_GPU, nthreads=NTHREADS)
    t = 0.0
    for _ in range(n):
        rc, t = orc.step(ig, b, t)
        assert rc == 0
    st = red["state"]
    assert st["t"] == t
    assert np.array_equal(vec(st["r"]), vec(b.r)) and np.array_equal(vec(st["v"]), vec(b.v))
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=dt, precision="fp64_exact", stage_exact=True) as sim:
        sim.launch_tries(n)
        sim.synchronize()
        out = sim.get_state(0)
        assert sim.info(0).t == t
    assert np.array_equal(vec(out.r), vec(st["r"])) and np.array_equal(vec(out.v), vec(st["v"]))


def test_red_gpu_rkf78_disk16384_adaptive(rg, orc, red_gpu):
    """The 16384-body disk, adaptive RKF7(8) at tol 1e-10, 30 steps from dt = 1 d."""
    s = rg.ic.config2()
    dt = 1.0 * rg.ic.K
    n = 30
    red = red_gpu.run(rg, s, "rkf78", dt, n, adaptive=True, tol=1e-10)
    b = obody(orc, s)
    ig = orc.make_integrator(orc.RKF78, dt, adaptive=True, tol=1e-10, sem=orc.SEM_GPU, nthreads=NTHREADS)
    t = 0.0
    hist = []
    for _ in range(n):
        rc, t = orc.step(ig, b, t)
        assert rc == 0
        hist.append((t, ig.dt_next, ig.n_tried, ig.n_passed, ig.n_failed))
    steps = red["steps"]
    for k in range(n):
        assert (steps["t"][k], steps["dt_next"][k]) == hist[k][:2], k
        assert (int(steps["tried"][k]), int(steps["passed"][k]), int(steps["failed"][k])) == hist[k][2:], k
    st = red["state"]
    assert np.array_equal(vec(st["r"]), vec(b.r)) and np.array_equal(vec(st["v"]), vec(b.v))
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=dt, precision="fp64_exact",
                stage_exact=True) as sim:
        for k in range(n):
            sim.step()
            info = sim.info(0)
            assert (info.n_tried, info.n_passed, info.n_failed) == hist[k][2:], k
            assert info.t == pytest.approx(hist[k][0], rel=1e-8)
        out = sim.get_state(0)
    print("disk16384 rkf78 adaptive 30 steps: fp64_exact bit-identical to red's GPU run: %s"
          % np.array_equal(vec(out.r), vec(st["r"])))
    assert np.allclose(vec(out.r), vec(st["r"]), rtol=1e-7, atol=1e-12)
    assert np.allclose(vec(out.v), vec(st["v"]), rtol=1e-7, atol=1e-12)


def planted_collisions(rg, orc, s):
    """s with planetesimal radii inflated until 50 .. n/8 pairs overlap at
    factor 1, plus two bodies inside the star's enlarged radius (red's GPU
    loop takes the star as i).  The pairs are counted with the oracle first:
    red's event buffer holds n records and is not bounds-checked."""
    n_si = s.n_SI
    R0 = s.p["radius"].copy()
    for g in (400.0, 600.0, 900.0, 1300.0, 2000.0):
        s.p["radius"][n_si:] = R0[n_si:] * g
        _, _, cnt = orc.check_collision(obody(orc, s), 0.0, 1.0, sem=orc.SEM_GPU, cap=s.n, nthreads=NTHREADS)
        if cnt >= 50:
            break
    for k in (n_si + 5, n_si + 11):
        d = 0.9 * (s.p["radius"][0] + s.p["radius"][k])
        s.r["x"][k], s.r["y"][k], s.r["z"][k] = s.r["x"][0] + d, s.r["y"][0], s.r["z"][0]
    _, ev, cnt = orc.check_collision(obody(orc, s), 0.0, 1.0, sem=orc.SEM_GPU, cap=s.n, nthreads=NTHREADS)
    assert 50 <= cnt <= s.n // 8, cnt
    return s, ev


def sorted_pairs(ev):
    k = np.lexsort((ev["idx2"], ev["idx1"], ev["event_name"]))
    return ev[k]


def test_red_gpu_collision_pairs_disk16384(rg, orc, red_gpu):
    s, ev_orc = planted_collisions(rg, orc, rg.ic.config2())
    ev_red = sorted_pairs(red_gpu.collisions(rg, s, 1.0))
    ev_orc = sorted_pairs(ev_orc)
    assert len(ev_red) == len(ev_orc)
    for f in ("event_name", "idx1", "idx2", "id1", "id2", "d"):
        assert np.array_equal(ev_red[f], ev_orc[f]), f
    assert (ev_red["idx1"] == 0).sum() + (ev_red["idx2"] == 0).sum() == 2      # the star pairs
    with rg.Sim(s, dt=0.01, collision_factor=1.0, event_capacity=s.n) as sim:
        ev_lib = sorted_pairs(sim.check_for_collision(cap=s.n))
    assert len(ev_lib) == len(ev_red)
    for f in ("event_name", "idx1", "idx2", "d"):
        assert np.array_equal(ev_lib[f], ev_red[f]), f
