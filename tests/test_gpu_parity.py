"""Parity of libredgb (through the C ABI, on cuda:0) with the oracle.

Tolerances:
  * FP64_EXACT gravity + stage_exact: bit-identical to the oracle's
    restatement of red's GPU kernels (no FMA, red's order).
  * FP64 step control uses pow(): CUDA's and glibc's pow may differ in the
    last bit, so adaptive trajectories are compared to 1e-10 relative and the
    step counters must be equal.
  * MIXED gravity: body-body pairs in FP32 -> per-body acceleration within
    2e-6 relative of the FP64 oracle for bodies without a star term, 1e-9 for
    the rest (the double-single star term, ~2e-14, dominates there).
  * Collision pairs: identical (integer work).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def obody(orc, s):
    return orc.Body(s.r, s.v, s.p, s.md, s.playing)


def vec(a):
    return np.stack([a["x"], a["y"], a["z"]], axis=1)


def small_disk(rg, n_pl=300, seed=1, n_tp=0):
    rng = np.random.Generator(np.random.MT19937(seed))
    return rg.ic.build_system(rng, pp_a=np.array([0.8, 1.0, 1.2, 1.4]), pp_mass=0.1 * rg.ic.EARTH_TO_SOLAR,
                              pl_a=rng.uniform(0.7, 1.5, n_pl), pl_mass=rg.ic.EARTH_TO_SOLAR / n_pl, n_tp=n_tp)


def test_gravity_fp64_exact_bitexact(rg, orc):
    s = small_disk(rg, n_pl=300, n_tp=7)
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=0.01, precision="fp64_exact", stage_exact=True) as sim:
        a = sim.calc_dydx(0, 1, 0.0)
    rc, ref = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU)
    assert rc == 0
    assert np.array_equal(vec(a), vec(ref))


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp32"])
def test_gravity_precisions(rg, orc, precision):
    s = small_disk(rg, n_pl=500, seed=3, n_tp=5)
    with rg.Sim(s, integrator="rkf78", dt=0.01, precision=precision) as sim:
        a = vec(sim.calc_dydx(0, 1, 0.0))
    _, ref = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU)
    ref = vec(ref)
    err = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    if precision == "fp64":
        assert err.max() < 1e-13
    else:
        # the star feels only FP32 pairs; every other body is dominated by the FP64 star term
        assert err[0] < 2e-6
        assert err[1:].max() < (1e-9 if precision == "mixed" else 5e-8)


def test_gravity_dense_mixed(rg, orc):
    s = small_disk(rg, n_pl=1000, seed=4).relabel_all_SI()
    with rg.Sim(s, dt=0.01, precision="mixed") as sim:
        a = vec(sim.calc_dydx(0, 1, 0.0))
    _, ref = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU)
    ref = vec(ref)
    err = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err[0] < 2e-6          # the star: FP32 pairs only
    assert err[1:].max() < 1e-8


@pytest.mark.parametrize("cluster", ["1", "0"])
def test_gravity_chunk_reduction_paths(rg, orc, monkeypatch, cluster):
    """The large bodies' sums over more than two source tiles are split into
    chunks: reduced through distributed shared memory within a thread-block
    cluster (the default when the launch fits the GPU at once) or through
    global partial records (REDGB_CLUSTER=0).  Both against the FP64 oracle
    with the MIXED tolerances: 2e-6 for the star (FP32 pairs only), 2e-9 for
    the bodies whose star term dominates."""
    monkeypatch.setenv("REDGB_CLUSTER", cluster)
    s = rg.ic.config2(seed=42, n_pp=8, n_pl=3000)
    with rg.Sim(s, dt=0.01, precision="mixed") as sim:
        a = vec(sim.calc_dydx(0, 1, 0.0))
    _, ref = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU)
    ref = vec(ref)
    err = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err[0] < 2e-6
    assert err[1:].max() < 2e-9, err[1:].max()


def test_velocity_derivative(rg):
    s = small_disk(rg, n_pl=50)
    with rg.Sim(s, dt=0.01) as sim:
        dv = sim.calc_dydx(0, 0, 0.0)
    assert np.array_equal(vec(dv), vec(s.v))


def test_drag(rg, orc):
    s = rg.ic.config3(n_pp=3, n_pl=200, seed=5)
    keys = rg.ic.gas_disk_config3()
    keys["time_dependence"] = "exponential"
    keys["t0"] = 0.5
    keys["e_folding_time"] = 3.0
    gas = np.array([rg.ic.gas_params(keys)], dtype=rg.types.GAS)
    t = 1.25 * 365.25 * rg.ic.K
    with rg.Sim(s, dt=0.01, precision="fp64_exact", stage_exact=True, gas=gas[0]) as sim:
        a = vec(sim.calc_dydx(0, 1, t))
    rc, ref = orc.calc_dydx(obody(orc, s), 1, t, gas=np.ascontiguousarray(gas, dtype=orc.GAS), sem=orc.SEM_GPU)
    ref = vec(ref)
    assert np.allclose(a, ref, rtol=1e-12, atol=0)
    _, grav = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU)
    nsi = s.n_SI
    assert np.abs(ref[nsi:] - vec(grav)[nsi:]).max() > 0.0   # drag acts


def test_drag_mixed(rg, orc):
    """MIXED evaluates the drag factor in FP32.  The drag part of the
    acceleration (with the gas disk minus without) follows the oracle's to
    1e-5 of itself plus the rounding of the sum (4e-16 of the acceleration);
    the drag is at most ~1e-5 of a body's acceleration here, so the whole
    acceleration keeps the mode's 1e-9."""
    s = rg.ic.config3(n_pp=3, n_pl=200, seed=5)
    keys = rg.ic.gas_disk_config3()
    keys["time_dependence"] = "exponential"
    keys["t0"] = 0.5
    keys["e_folding_time"] = 3.0
    gas = np.array([rg.ic.gas_params(keys)], dtype=rg.types.GAS)
    t = 1.25 * 365.25 * rg.ic.K
    with rg.Sim(s, dt=0.01, precision="mixed", gas=gas[0]) as sim:
        a = vec(sim.calc_dydx(0, 1, t))
    with rg.Sim(s, dt=0.01, precision="mixed") as sim:
        a0 = vec(sim.calc_dydx(0, 1, t))
    rc, ref = orc.calc_dydx(obody(orc, s), 1, t, gas=np.ascontiguousarray(gas, dtype=orc.GAS), sem=orc.SEM_GPU)
    ref = vec(ref)
    _, grav = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU)
    nsi = s.n_SI
    drag, dref = (a - a0)[nsi:], (ref - vec(grav))[nsi:]
    bound = 1e-5 * np.linalg.norm(dref, axis=1) + 4e-16 * np.linalg.norm(a[nsi:], axis=1)
    assert np.all(np.linalg.norm(drag - dref, axis=1) <= bound)
    err = np.linalg.norm(a[nsi:] - ref[nsi:], axis=1) / np.linalg.norm(ref[nsi:], axis=1)
    assert err.max() < 1e-9


def run_oracle(orc, s, kind, dt, nsteps, adaptive, tol=0.0, gas=None, eftp=False):
    b = obody(orc, s)
    okind = {"euler": orc.EULER, "rk2": orc.RK2, "rk4": orc.RK4, "rkf78": orc.RKF78}[kind]
    ig = orc.make_integrator(okind, dt, adaptive=adaptive, tol=tol, error_check_for_tp=eftp, sem=orc.SEM_GPU)
    t = 0.0
    hist = []
    for _ in range(nsteps):
        rc, t = orc.step(ig, b, t, gas=gas)
        assert rc == 0
        hist.append((t, ig.dt_did, ig.dt_next, ig.n_tried, ig.n_passed, ig.n_failed))
    return b, hist


@pytest.mark.parametrize("kind,adaptive", [("rk4", False), ("rkf78", False), ("euler", False), ("rk2", False)])
def test_fixed_step_bitexact(rg, orc, kind, adaptive):
    s = small_disk(rg, n_pl=200, seed=7, n_tp=3)
    dt = {"rk4": 0.5, "rkf78": 4.0, "euler": 0.05, "rk2": 0.2}[kind] * rg.ic.K
    n = 12
    ref, hist = run_oracle(orc, s, kind, dt, n, adaptive)
    with rg.Sim(s, integrator=kind, adaptive=adaptive, dt=dt, precision="fp64_exact", stage_exact=True) as sim:
        for k in range(n):
            d = sim.step()
            assert d == hist[k][1]
        out = sim.get_state(0)
        info = sim.info(0)
    assert info.t == hist[-1][0]
    assert np.array_equal(vec(out.r), vec(ref.r))
    assert np.array_equal(vec(out.v), vec(ref.v))


@pytest.mark.parametrize("kind", ["rk2", "rk4", "rkf78"])
def test_fixed_step_with_time_dependent_drag(rg, orc, kind):
    """Stage times t + c_s dt reach the gas disk's time dependence (exponential
    decay after t0); the trajectory with drag follows the oracle's.  Drag uses
    pow / exp, whose CUDA and glibc roundings may differ in the last bit, so
    the comparison is to 1e-12 relative, not bit for bit."""
    s = rg.ic.config3(n_pp=3, n_pl=120, seed=9)
    keys = rg.ic.gas_disk_config3()
    keys["time_dependence"] = "exponential"
    keys["t0"] = 0.0
    keys["e_folding_time"] = 0.05
    gas = np.array([rg.ic.gas_params(keys)], dtype=rg.types.GAS)
    dt = {"rk2": 0.2, "rk4": 0.5, "rkf78": 4.0}[kind] * rg.ic.K
    n = 8
    ref, hist = run_oracle(orc, s, kind, dt, n, False, gas=np.ascontiguousarray(gas, dtype=orc.GAS))
    with rg.Sim(s, integrator=kind, adaptive=False, dt=dt, precision="fp64_exact", stage_exact=True,
                gas=gas[0]) as sim:
        for k in range(n):
            assert sim.step() == hist[k][1]
        out = sim.get_state(0)
    for got, want in ((vec(out.r), vec(ref.r)), (vec(out.v), vec(ref.v))):
        err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
        assert err.max() < 1e-12, err.max()


@pytest.mark.parametrize("kind,tol,eftp", [("rkf78", 1e-10, False), ("rk4", 1e-10, False), ("rkf78", 1e-12, True)])
def test_adaptive_matches_oracle(rg, orc, kind, tol, eftp):
    s = small_disk(rg, n_pl=150, seed=8, n_tp=4)
    dt = 5.0 * rg.ic.K
    n = 15
    ref, hist = run_oracle(orc, s, kind, dt, n, True, tol, eftp=eftp)
    with rg.Sim(s, integrator=kind, adaptive=True, tolerance=tol, dt=dt, precision="fp64_exact",
                stage_exact=True, error_check_for_tp=eftp) as sim:
        for k in range(n):
            sim.step()
            info = sim.info(0)
            assert (info.n_tried, info.n_passed, info.n_failed) == hist[k][3:], k
            # CUDA's and glibc's pow() may round differently in the last bit; the
            # embedded error estimate (a difference of nearly equal stage sums)
            # magnifies such 1-ulp differences, so step sizes are compared loosely
            assert info.t == pytest.approx(hist[k][0], rel=1e-9)
            assert info.dt_next == pytest.approx(hist[k][2], rel=1e-5)
        out = sim.get_state(0)
    assert np.allclose(vec(out.r), vec(ref.r), rtol=1e-8, atol=1e-12)
    assert np.allclose(vec(out.v), vec(ref.v), rtol=1e-8, atol=1e-12)


@pytest.mark.parametrize("precision,bound", [("mixed", 1e-10), ("fp32", 1e-8), ("fp64", 1e-12)])
def test_trajectory_close_to_fp64(rg, orc, precision, bound):
    # fixed step, so that both runs sample the same times
    s = small_disk(rg, n_pl=300, seed=9)
    dt = 2.0 * rg.ic.K
    n = 30
    ref, _ = run_oracle(orc, s, "rkf78", dt, n, False)
    with rg.Sim(s, integrator="rkf78", adaptive=False, dt=dt, precision=precision) as sim:
        for _ in range(n):
            sim.step()
        out = sim.get_state(0)
    rel = np.linalg.norm(vec(out.r) - vec(ref.r), axis=1) / np.linalg.norm(vec(ref.r), axis=1)
    assert rel[1:].max() < bound


def test_adaptive_mixed_energy(rg, orc):
    s = small_disk(rg, n_pl=300, seed=9)
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=5.0 * rg.ic.K, precision="mixed") as sim:
        E0 = sim.energy_interacting(0)
        for _ in range(40):
            sim.step()
        E1 = sim.energy_interacting(0)
        info = sim.info(0)
    assert info.n_passed == 40
    assert abs((E1[0] - E0[0]) / E0[0]) < 1e-9
    assert np.allclose(E1[1:], E0[1:], rtol=1e-10)


def collide_disk(rg):
    s = small_disk(rg, n_pl=120, seed=12, n_tp=2)
    r, p = s.r, s.p
    R = p["radius"]

    v = s.v

    def place(j, i, frac):
        # j next to i, moving with i, so that the pair still overlaps after a short step
        d = frac * (R[i] + R[j])
        r["x"][j], r["y"][j], r["z"][j] = r["x"][i] + d, r["y"][i], r["z"][i]
        v["x"][j], v["y"][j], v["z"][j] = v["x"][i], v["y"][i], v["z"][i]

    place(10, 9, 0.6)
    place(11, 10, 0.5)
    p["mass"][13] = 3.0 * p["mass"][12]
    place(13, 12, 0.9)
    place(s.n - 1, 2, 0.4)
    place(6, 0, 0.5)
    place(100, 70, 0.9)
    return s


def keys(ev):
    return [(int(e["event_name"]), int(e["idx1"]), int(e["idx2"])) for e in ev]


def test_collision_pairs_identical(rg, orc):
    s = collide_disk(rg)
    with rg.Sim(s, dt=0.01, collision_factor=1.0) as sim:
        ev = sim.check_for_collision()
    _, ref, _ = orc.check_collision(obody(orc, s), 0.0, 1.0, sem=orc.SEM_GPU)
    assert len(ref) >= 6
    assert keys(ev) == keys(ref)
    assert np.array_equal(ev["d"], ref["d"])


def test_collision_factor_and_merge_during_run(rg, orc):
    s = collide_disk(rg)
    dt = 0.5 * rg.ic.K
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=dt, precision="fp64_exact", stage_exact=True,
                collision_factor=1.0) as sim:
        sim.launch_tries(1)
        n_active, n_halted = sim.synchronize()
        assert n_halted == 1
        handled = sim.handle_events()
        out = sim.get_state(0)
        info = sim.info(0)
    # oracle: one RK4 step, GPU-semantics check on the new state, red's merge
    b = obody(orc, s)
    ig = orc.make_integrator(orc.RK4, dt, sem=orc.SEM_GPU)
    rc, t = orc.step(ig, b, 0.0)
    rc, ev, n = orc.check_collision(b, t, 1.0, sem=orc.SEM_GPU)
    rc, sp = orc.handle_collision(b, ev)
    assert keys(handled) == keys(sp)
    for f in ["p1", "p2", "ps", "rs", "vs", "r1", "r2", "v1", "v2"]:
        assert np.array_equal(np.ascontiguousarray(handled[f]).view(np.uint8),
                              np.ascontiguousarray(sp[f]).view(np.uint8)), f
    assert np.array_equal(vec(out.r), vec(b.r))
    assert np.array_equal(out.md["id"], b.md["id"])
    assert list(info.inactive) == list(b.inactive)
    assert info.n_collision[0] == len(sp)


def test_ejection_hit_centrum(rg, orc):
    s = small_disk(rg, n_pl=60, seed=13)
    for c in "xyz":
        s.r[c][5] *= 30.0
        s.r[c][8] *= 0.05
    with rg.Sim(s, dt=0.01, ejection=20.0, hit_centrum=0.1) as sim:
        ev = sim.check_for_ejection_hit_centrum()
    _, ref, _ = orc.check_ejection_hit_centrum(obody(orc, s), 0.0, 20.0, 0.1)
    assert sorted(keys(ev)) == sorted(keys(ref))


def test_integrals(rg, orc):
    s = collide_disk(rg)
    s.md["id"][4] *= -1
    with rg.Sim(s, dt=0.01) as sim:
        I = sim.calc_integral(0)
        Ei = sim.energy_interacting(0)
    ref = orc.calc_integral(obody(orc, s))
    assert np.allclose(I, ref, rtol=1e-12, atol=1e-18)
    refi = orc.energy_interacting(obody(orc, s))
    assert np.allclose(Ei, refi, rtol=1e-12, atol=1e-20)


def test_rebuild_vectors_after_merges(rg, orc):
    s = collide_disk(rg)
    dt = 0.5 * rg.ic.K
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=dt, precision="fp64_exact", stage_exact=True,
                collision_factor=1.0) as sim:
        sim.launch_tries(1)
        sim.synchronize()
        sim.handle_events()
        sim.rebuild_vectors()
        out = sim.get_state(0)
        info = sim.info(0)
        sim.step()     # integrates on after the compaction
    b = obody(orc, s)
    ig = orc.make_integrator(orc.RK4, dt, sem=orc.SEM_GPU)
    rc, t = orc.step(ig, b, 0.0)
    rc, ev, n = orc.check_collision(b, t, 1.0, sem=orc.SEM_GPU)
    orc.handle_collision(b, ev)
    orc.rebuild_vectors(b)
    assert out.n == b.n
    assert list(info.playing) == list(b.playing)
    assert list(info.removed) == list(b.removed)
    assert np.array_equal(vec(out.r), vec(b.r))
    assert np.array_equal(out.md["id"], b.md["id"])


def test_ensemble_equals_single_systems(rg):
    systems = [small_disk(rg, n_pl=50 + 37 * k, seed=20 + k) for k in range(5)]
    dt = 2.0 * rg.ic.K
    kw = dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=dt, precision="fp64_exact", stage_exact=True)
    singles = []
    for s in systems:
        with rg.Sim(s, **kw) as sim:
            for _ in range(6):
                sim.step()
            singles.append((sim.get_state(0), sim.info(0).t))
    with rg.Sim(systems, **kw) as sim:
        for _ in range(6):
            sim.step()
        for k in range(len(systems)):
            st = sim.get_state(k)
            assert sim.info(k).t == singles[k][1]
            assert np.array_equal(vec(st.r), vec(singles[k][0].r))


@pytest.mark.parametrize("factor", [300.0, 2000.0])
def test_collision_many_pairs_grid(rg, orc, factor):
    # enlarged radii make many planetesimal pairs overlap: the spatial-hash grid
    # (small bodies) and the brute-force pass (SI bodies) must find red's exact pair set
    systems = [rg.ic.config1(seed=31 + k, n_pl=1500 + 500 * k) for k in range(3)]
    with rg.Sim(systems, dt=0.01, collision_factor=factor, event_capacity=1 << 16) as sim:
        ev = sim.check_for_collision(cap=1 << 16)
    got = {}
    for e in ev:
        got.setdefault(len(got), None)
    n_ref = 0
    start = 0
    for k, s in enumerate(systems):
        _, ref, n = orc.check_collision(obody(orc, s), 0.0, factor, sem=orc.SEM_GPU, cap=1 << 16)
        assert n == len(ref)
        n_ref += n
        mine = ev[start:start + n]
        start += n
        assert keys(mine) == keys(ref), k
        assert np.array_equal(mine["d"], ref["d"])
    assert len(ev) == n_ref
    assert n_ref > 50


def pinned_copy(rg, s):
    """A System whose r, v, p, md arrays live in page-locked host memory."""
    torch = pytest.importorskip("torch")
    out = rg.types.System(s.r.copy(), s.v.copy(), s.p.copy(), s.md.copy(), s.playing.copy())
    keep = []
    for f, t in (("r", rg.types.VAR4), ("v", rg.types.VAR4), ("p", rg.types.PARAM), ("md", rg.types.BMD)):
        buf = torch.from_numpy(getattr(s, f).copy().view(np.uint8)).pin_memory()
        keep.append(buf)
        setattr(out, f, buf.numpy().view(t))
    out._pinned = keep
    return out


def test_state_transfer_pinned_equals_pageable(rg):
    """red_get_state / red_set_state read and write pinned caller arrays from the
    kernel itself and pageable ones through the staging buffer: same bytes."""
    s = small_disk(rg, n_pl=500, seed=4)
    kw = dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K, precision="mixed")
    with rg.Sim(s, **kw) as sim:
        for _ in range(3):
            sim.step()
        a = sim.get_state(0)
        b = pinned_copy(rg, a)
        for f in ("r", "v", "p", "md"):
            getattr(b, f)[:] = 0
        sim.get_state(0, out=b)
        for f in ("r", "v", "p"):
            assert getattr(a, f).tobytes() == getattr(b, f).tobytes(), f
        for f in a.md.dtype.names:   # field by field: the records' padding is the caller's
            assert np.array_equal(a.md[f], b.md[f]), f
    moved = small_disk(rg, n_pl=500, seed=4)
    moved.r["x"][5:40] += 1e-7
    moved.v["y"][10:20] *= 1.0 + 1e-9
    moved.p["radius"][30:50] *= 1.5
    ends = []
    for src in (moved, pinned_copy(rg, moved)):
        with rg.Sim(s, **kw) as sim:
            sim.set_state(0, src, parts="rvp")
            for _ in range(3):
                sim.step()
            ends.append(sim.get_state(0))
    for f in ("r", "v", "p"):
        assert getattr(ends[0], f).tobytes() == getattr(ends[1], f).tobytes(), f


@pytest.mark.parametrize("precision,bound", [("mixed", 1e-8), ("fp32", 5e-7)])
def test_gravity_packed_pairs(rg, orc, monkeypatch, precision, bound):
    """Plans of many waves whose tiles hold 2 sinks per thread take the packed
    FP32-pair instance (sources in pairs, add / mul / fma .f32x2).  An all-SI
    disk of 6017 bodies (source chunks of odd length, so the last pair of a
    tile is padded) against the FP64 oracle with the all-SI tolerances (2e-6
    for the star, FP32 pairs only; `bound` for the rest), and against the
    scalar instance (REDGB_PACKED=0) to the same bound."""
    s = rg.ic.config2(seed=44, n_pp=16, n_pl=6000).relabel_all_SI()
    out = {}
    for packed in ("1", "0"):
        monkeypatch.setenv("REDGB_PACKED", packed)
        with rg.Sim(s, dt=0.01, precision=precision) as sim:
            out[packed] = (vec(sim.calc_dydx(0, 1, 0.0)), sim.plan_info())
    assert out["1"][1]["packed"] and not out["0"][1]["packed"]
    _, ref = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU, nthreads=16)
    ref = vec(ref)
    for packed in ("1", "0"):
        a = out[packed][0]
        err = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert err[0] < 2e-6 and err[1:].max() < bound, (packed, err[0], err[1:].max())
    d = np.linalg.norm(out["1"][0] - out["0"][0], axis=1) / np.linalg.norm(ref, axis=1)
    assert d[1:].max() < bound


@pytest.mark.parametrize("precision,bound", [("mixed", 1e-8), ("fp32", 5e-7)])
def test_gravity_packed_pairs_streamed(rg, orc, monkeypatch, precision, bound):
    """The packed instance with chunks longer than the two-tile staging
    buffer: each prefetched tile goes straight into the pair records of the
    other of two buffers.  An all-SI disk of 16401 bodies, whose heuristic
    plan cuts every tile's sources into ~14 chunks of nine tiles (the last
    chunk 273 sources, so its last tile has an odd count and a padded pair),
    against the FP64 oracle and the scalar instance as in
    test_gravity_packed_pairs."""
    s = rg.ic.config2(seed=45, n_pp=16, n_pl=16384).relabel_all_SI()
    out = {}
    for packed in ("1", "0"):
        monkeypatch.setenv("REDGB_PACKED", packed)
        with rg.Sim(s, dt=0.01, precision=precision) as sim:
            out[packed] = (vec(sim.calc_dydx(0, 1, 0.0)), sim.plan_info())
    info = out["1"][1]
    tiles = (s.n + 31) // 32
    assert info["packed"] and info["n_items"] <= 20 * tiles   # chunks of > 2 tiles of 128 sources
    _, ref = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU, nthreads=16)
    ref = vec(ref)
    for packed in ("1", "0"):
        a = out[packed][0]
        err = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert err[0] < 2e-6 and err[1:].max() < bound, (packed, err[0], err[1:].max())
    d = np.linalg.norm(out["1"][0] - out["0"][0], axis=1) / np.linalg.norm(ref, axis=1)
    assert d[1:].max() < bound
