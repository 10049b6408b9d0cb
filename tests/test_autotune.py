"""red_autotune: the launch-plan search (red's own precedent is its
thread-per-block search, pp_disk::benchmark, src/red.cuda/pp_disk.cu:553-611).

The search integrates real tries of every candidate plan from a snapshot of
the live state and restores it: the state, the time and the counters after
the call are bit-identical to those before.  The tuned plan changes only how
the FP32 pair sums are grouped (chunks of whole source tiles, the same
double-single accumulation), so a MIXED trajectory under it agrees with the
untuned one to 1e-12 relative after 20 steps; the red-exact mode has one plan
and stays bit-identical to the oracle.  A default plan that reduces through a
thread-block cluster is among the candidates timed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def vec(a):
    return np.stack([a["x"], a["y"], a["z"]], axis=1)


def test_autotune_leaves_the_state_unchanged(rg):
    s = rg.ic.config2(seed=42, n_pp=8, n_pl=3000)
    with rg.Sim(s, dt=1.0 * rg.ic.K, precision="mixed", collision_factor=1.0) as sim:
        for _ in range(3):
            sim.step()
        before, ib = sim.get_state(0), sim.info(0)
        plan = sim.autotune()
        after, ia = sim.get_state(0), sim.info(0)
    assert plan["candidates"] >= 6 and plan["ms_per_try"] > 0.0
    assert (ia.t, ia.n_tried, ia.n_passed, ia.dt_next) == (ib.t, ib.n_tried, ib.n_passed, ib.dt_next)
    assert np.array_equal(vec(after.r), vec(before.r)) and np.array_equal(vec(after.v), vec(before.v))


def test_tuned_plan_follows_the_untuned_trajectory(rg):
    s = rg.ic.config2(seed=43, n_pp=8, n_pl=3000)
    out = []
    for tune in (False, True):
        with rg.Sim(s, integrator="rkf78", adaptive=False, dt=2.0 * rg.ic.K, precision="mixed") as sim:
            if tune:
                sim.autotune()
            for _ in range(20):
                sim.step()
            out.append(vec(sim.get_state(0).r))
    scale = np.linalg.norm(out[0], axis=1).max()
    assert np.abs(out[1] - out[0]).max() <= 1e-12 * scale


def test_autotune_ensemble_and_exact_mode(rg, orc):
    systems = [rg.ic.config1(seed=50 + k, n_pl=400 + 300 * k) for k in range(3)]
    with rg.Sim(systems, dt=1.0 * rg.ic.K, precision="mixed") as sim:
        plan = sim.autotune()
        sim.step()
    assert plan["candidates"] >= 6
    s = systems[1]
    dt = 0.5 * rg.ic.K
    b = orc.Body(s.r, s.v, s.p, s.md, s.playing)
    ig = orc.make_integrator(orc.RK4, dt, sem=orc.SEM_GPU)
    t = 0.0
    for _ in range(5):
        _, t = orc.step(ig, b, t)
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=dt, precision="fp64_exact") as sim:
        plan = sim.autotune()
        for _ in range(5):
            sim.step()
        out = sim.get_state(0)
    assert plan["candidates"] == 0
    assert np.array_equal(vec(out.r), vec(b.r)) and np.array_equal(vec(out.v), vec(b.v))


def test_autotune_times_the_cluster_plan(rg):
    """The 2053-body disk's default plan reduces its large-body chunks in a
    thread-block cluster (16 % faster per try than global records there); the
    search times that plan first and keeps it."""
    s = rg.ic.config1()
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=0.5 * rg.ic.K, precision="mixed") as sim:
        assert sim.plan_info()["cluster"]
        plan = sim.autotune()
    assert plan["cluster"] and plan["chunk"] == 0
    assert plan["ms_per_try"] <= plan["ms_per_try_default"]
