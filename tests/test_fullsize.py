"""The bench's workloads at their full sizes.

Against the oracle (its OpenMP build on the host's cores finishes each case
in seconds):
* the 2053-body disk over its whole length (fixed-step RK4, dt = 0.5 d, 2000
  steps): FP64_EXACT bit-identical; MIXED within 2e-8 relative in position
  (largest over the bodies; median 1e-10).
* the 16384-body disk, adaptive RKF7(8) at tol 1e-10, 50 steps: FP64_EXACT
  step counters equal at every step, t to 1e-8 and positions to 1e-7 (the
  step-size power is the nearest double, the C library's pow misrounds about
  1 call in 1000, and the error estimate magnifies such a 1-ulp difference);
  fixed-step RKF7(8) over 50 steps of 2 d: MIXED within 1e-8 relative
  (largest over the bodies; median 1e-10).
* the gas-drag disk (65536 bodies), 5 adaptive steps with drag: FP64_EXACT
  counters equal and positions to 1e-7; MIXED at fixed step within 1e-8
  (median 1e-10).
* 8 disks sampled from the 512-disk ensemble, run together with the other
  504: FP64_EXACT counters equal and positions to 1e-7 against each disk run
  alone by the oracle.
* collision pairs of the 16384-body disk through the spatial hash at full
  density (hundreds of pairs): identical to the oracle's.

Size-independent properties where the oracle is not needed:
* the 16384-body disk (MIXED, adaptive RKF7(8) at tol 1e-10; collisions off,
  since a perfect merge changes E by design): energy over the interacting
  pairs conserved to |dE/E| < 1e-9 and the angular momentum to 1e-10 over
  300 tries, the metric's accuracy bar.
* the 512-disk ensemble (1.08 M bodies): the same bar for every disk after 30
  tries, and the ensemble's counters consistent (tried = passed + failed).
* the same disk with every pair interacting: the same bar after 8 tries.
* the 2053-body disk (RK4 fixed step): MIXED against FP64 after 100 steps,
  1e-10 relative in position (the precision modes agree at full size).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def vec(a):
    return np.stack([a["x"], a["y"], a["z"]], axis=1)


def conserved(sim, k, E0):
    E1 = sim.energy_interacting(k)
    dE = abs((E1[0] - E0[0]) / E0[0])
    dC = np.abs(E1[1:] - E0[1:]).max() / np.abs(E0[1:]).max()
    return dE, dC


def test_c2_conserves_energy_and_angular_momentum(rg):
    s = rg.ic.config2()
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K, precision="mixed") as sim:
        E0 = sim.energy_interacting(0)
        sim.launch_tries(300)
        sim.synchronize()
        dE, dC = conserved(sim, 0, E0)
        info = sim.info(0)
    assert info.n_passed > 200 and info.n_tried == info.n_passed + info.n_failed
    assert dE < 1e-9, dE
    assert dC < 1e-10, dC


def test_c4_ensemble_conserves_energy(rg):
    systems = rg.ic.config4()
    with rg.Sim(systems, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K,
                precision="mixed") as sim:
        E0 = [sim.energy_interacting(k) for k in range(len(systems))]
        sim.launch_tries(30)
        sim.synchronize()
        worst = 0.0
        for k in range(len(systems)):
            dE, dC = conserved(sim, k, E0[k])
            worst = max(worst, dE)
            assert dC < 1e-10, (k, dC)
            info = sim.info(k)
            assert info.n_passed > 0 and info.n_tried == info.n_passed + info.n_failed
    assert worst < 1e-9, worst


def test_dense_conserves_energy(rg):
    s = rg.ic.config2().relabel_all_SI()
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K,
                precision="mixed") as sim:
        E0 = sim.energy_interacting(0)
        sim.launch_tries(8)
        sim.synchronize()
        dE, dC = conserved(sim, 0, E0)
    assert dE < 1e-9, dE
    assert dC < 1e-10, dC


def test_c1_mixed_matches_fp64(rg):
    s = rg.ic.config1()
    out = {}
    for prec in ("mixed", "fp64"):
        with rg.Sim(s, integrator="rk4", adaptive=False, dt=0.5 * rg.ic.K, precision=prec) as sim:
            sim.launch_tries(100)
            sim.synchronize()
            out[prec] = vec(sim.get_state(0).r)
    scale = np.linalg.norm(out["fp64"], axis=1).max()
    assert np.abs(out["mixed"] - out["fp64"]).max() < 1e-10 * scale


NTHREADS = 16


def obody(orc, s):
    return orc.Body(s.r, s.v, s.p, s.md, s.playing)


def oracle_run(orc, s, kind, dt, n, adaptive=False, tol=1e-10, gas=None):
    b = obody(orc, s)
    ig = orc.make_integrator(kind, dt, adaptive=adaptive, tol=tol, sem=orc.SEM_GPU, nthreads=NTHREADS)
    t = 0.0
    hist = []
    for _ in range(n):
        rc, t = orc.step(ig, b, t, gas=gas)
        assert rc == 0
        hist.append((t, ig.n_tried, ig.n_passed, ig.n_failed))
    return b, hist


def rel_pos(a, b):
    return (np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)).max()


def rel_med(a, b):
    return float(np.median(np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)))


def test_c1_full_length_matches_oracle(rg, orc):
    s = rg.ic.config1()
    dt = 0.5 * rg.ic.K
    n = 2000
    b, hist = oracle_run(orc, s, orc.RK4, dt, n)
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=dt, precision="fp64_exact", stage_exact=True) as sim:
        sim.launch_tries(n)
        sim.synchronize()
        out = sim.get_state(0)
        assert sim.info(0).t == hist[-1][0]
    assert np.array_equal(vec(out.r), vec(b.r)) and np.array_equal(vec(out.v), vec(b.v))
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=dt, precision="mixed") as sim:
        sim.launch_tries(n)
        sim.synchronize()
        out = sim.get_state(0)
    err, med = rel_pos(vec(out.r)[1:], vec(b.r)[1:]), rel_med(vec(out.r)[1:], vec(b.r)[1:])
    print("disk2053 rk4 2000 steps: mixed vs oracle, relative position error max %.3e median %.3e" % (err, med))
    assert err < 2e-8 and med < 1e-10, (err, med)


def test_c2_adaptive_matches_oracle(rg, orc):
    s = rg.ic.config2()
    dt = 1.0 * rg.ic.K
    n = 50
    b, hist = oracle_run(orc, s, orc.RKF78, dt, n, adaptive=True)
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=dt, precision="fp64_exact",
                stage_exact=True) as sim:
        for k in range(n):
            sim.step()
            info = sim.info(0)
            assert (info.n_tried, info.n_passed, info.n_failed) == hist[k][1:], k
            assert info.t == pytest.approx(hist[k][0], rel=1e-8)
        out = sim.get_state(0)
    print("disk16384 rkf78 adaptive 50 steps, fp64_exact: t %.17g (oracle %.17g), bit-identical state: %s"
          % (info.t, hist[-1][0], np.array_equal(vec(out.r), vec(b.r))))
    assert np.allclose(vec(out.r), vec(b.r), rtol=1e-7, atol=1e-12)
    assert np.allclose(vec(out.v), vec(b.v), rtol=1e-7, atol=1e-12)
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=dt, precision="mixed") as sim:
        for k in range(n):
            sim.step()
        info = sim.info(0)
        out = sim.get_state(0)
    print("disk16384 rkf78 adaptive 50 steps: mixed tried %d (oracle %d), t %.17g (oracle %.17g), "
          "max relative position error %.3e" % (info.n_tried, hist[-1][1], info.t, hist[-1][0],
                                                rel_pos(vec(out.r)[1:], vec(b.r)[1:])))


def test_c2_fixed_step_mixed_matches_oracle(rg, orc):
    s = rg.ic.config2()
    dt = 2.0 * rg.ic.K
    n = 50
    b, _ = oracle_run(orc, s, orc.RKF78, dt, n)
    with rg.Sim(s, integrator="rkf78", adaptive=False, dt=dt, precision="mixed") as sim:
        sim.launch_tries(n)
        sim.synchronize()
        out = sim.get_state(0)
    err, med = rel_pos(vec(out.r)[1:], vec(b.r)[1:]), rel_med(vec(out.r)[1:], vec(b.r)[1:])
    print("disk16384 rkf78 fixed 50 x 2 d: mixed vs oracle, relative position error max %.3e median %.3e"
          % (err, med))
    assert err < 1e-8 and med < 1e-10, (err, med)


def test_c3_gas_drag_matches_oracle(rg, orc):
    s = rg.ic.config3()
    keys = rg.ic.gas_disk_config3()
    gas = np.array([rg.ic.gas_params(keys)], dtype=rg.types.GAS)
    ogas = np.ascontiguousarray(gas, dtype=orc.GAS)
    dt = 1.0 * rg.ic.K
    n = 5
    b, hist = oracle_run(orc, s, orc.RKF78, dt, n, adaptive=True, gas=ogas)
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=dt, precision="fp64_exact",
                stage_exact=True, gas=gas[0]) as sim:
        for k in range(n):
            sim.step()
            info = sim.info(0)
            assert (info.n_tried, info.n_passed, info.n_failed) == hist[k][1:], k
            assert info.t == pytest.approx(hist[k][0], rel=1e-8)
        out = sim.get_state(0)
    print("disk65536 gas rkf78 adaptive 5 steps, fp64_exact: t %.17g (oracle %.17g), bit-identical state: %s"
          % (info.t, hist[-1][0], np.array_equal(vec(out.r), vec(b.r))))
    assert np.allclose(vec(out.r), vec(b.r), rtol=1e-7, atol=1e-12)
    b, _ = oracle_run(orc, s, orc.RKF78, dt, n, gas=ogas)
    with rg.Sim(s, integrator="rkf78", adaptive=False, dt=dt, precision="mixed", gas=gas[0]) as sim:
        sim.launch_tries(n)
        sim.synchronize()
        out = sim.get_state(0)
    err, med = rel_pos(vec(out.r)[1:], vec(b.r)[1:]), rel_med(vec(out.r)[1:], vec(b.r)[1:])
    print("disk65536 gas rkf78 fixed 5 x 1 d: mixed vs oracle, relative position error max %.3e median %.3e"
          % (err, med))
    assert err < 1e-8 and med < 1e-10, (err, med)


def test_c4_sampled_disks_match_oracle(rg, orc):
    systems = rg.ic.config4()
    dt = 1.0 * rg.ic.K
    n = 8
    sample = np.random.Generator(np.random.MT19937(4)).choice(len(systems), 8, replace=False)
    with rg.Sim(systems, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=dt, precision="fp64_exact",
                stage_exact=True) as sim:
        for _ in range(n):
            sim.step()
        got = {int(k): (sim.get_state(int(k)), sim.info(int(k))) for k in sample}
    exact = 0
    for k in sample:
        b, hist = oracle_run(orc, systems[k], orc.RKF78, dt, n, adaptive=True)
        st, info = got[int(k)]
        assert (info.n_tried, info.n_passed, info.n_failed) == hist[-1][1:], k
        assert info.t == pytest.approx(hist[-1][0], rel=1e-8)
        assert np.allclose(vec(st.r), vec(b.r), rtol=1e-7, atol=1e-12), k
        assert np.allclose(vec(st.v), vec(b.v), rtol=1e-7, atol=1e-12), k
        exact += int(np.array_equal(vec(st.r), vec(b.r)))
    print("ensemble of 512 disks, 8 sampled, fp64_exact: %d of 8 bit-identical to the oracle" % exact)


def test_c2_collision_pairs_full_density(rg, orc):
    """Planetesimal radii inflated until hundreds of pairs overlap: the hash
    grid's cells grow with the largest collision distance, so this runs the
    grid at the disk's own density."""
    s = rg.ic.config2()
    n_si = s.n_SI
    R0 = s.p["radius"].copy()
    for g in (1000.0, 1400.0, 2000.0, 2800.0, 4000.0):
        s.p["radius"][n_si:] = R0[n_si:] * g
        _, ev_orc, cnt = orc.check_collision(obody(orc, s), 0.0, 1.0, sem=orc.SEM_GPU, cap=s.n,
                                             nthreads=NTHREADS)
        if cnt >= 200:
            break
    assert cnt >= 200, cnt
    with rg.Sim(s, dt=0.01, collision_factor=1.0, event_capacity=s.n) as sim:
        ev = sim.check_for_collision(cap=s.n)

    def srt(e):
        return e[np.lexsort((e["idx2"], e["idx1"]))]
    ev, ev_orc = srt(ev), srt(ev_orc)
    assert len(ev) == len(ev_orc)
    for f in ("event_name", "idx1", "idx2", "d"):
        assert np.array_equal(ev[f], ev_orc[f]), f
