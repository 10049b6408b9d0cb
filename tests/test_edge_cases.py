"""Edge cases of the path, through the C ABI on cuda:0, against the oracle.

Degenerate systems (a lone star, a star and one body, a disk without
protoplanets, test particles only), inactive bodies (id < 0) inside the
source and sink ranges, and a ragged ensemble that mixes all of them with a
large disk.  FP64_EXACT runs compare bit for bit with the oracle; the MIXED
runs use the MIXED tolerances (2e-6 for the star, which feels FP32 pairs
only; 1e-9 for bodies dominated by the double-single star term).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def obody(orc, s):
    return orc.Body(s.r, s.v, s.p, s.md, s.playing)


def vec(a):
    return np.stack([a["x"], a["y"], a["z"]], axis=1)


def disk(rg, n_pp=4, n_pl=200, n_tp=0, seed=3):
    rng = np.random.Generator(np.random.MT19937(seed))
    pp_a = 0.8 + 0.2 * np.arange(n_pp)
    return rg.ic.build_system(rng, pp_a=pp_a, pp_mass=0.1 * rg.ic.EARTH_TO_SOLAR,
                              pl_a=rng.uniform(0.7, 1.5, n_pl), pl_mass=rg.ic.EARTH_TO_SOLAR / max(n_pl, 1),
                              n_tp=n_tp)


def fixed_run(rg, orc, s, n=6, dt_days=0.5):
    dt = dt_days * rg.ic.K
    b = obody(orc, s)
    ig = orc.make_integrator(orc.RK4, dt, sem=orc.SEM_GPU)
    t = 0.0
    for _ in range(n):
        rc, t = orc.step(ig, b, t)
        assert rc == 0
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=dt, precision="fp64_exact", stage_exact=True) as sim:
        for _ in range(n):
            sim.step()
        out = sim.get_state(0)
        assert sim.info(0).t == t
    return out, b


def test_lone_star_is_finished(rg):
    """run_simulation integrates while more than one body is active (main.cu:471):
    a lone star is a finished system; red_step leaves it where it is."""
    s = disk(rg, n_pp=0, n_pl=0)
    with rg.Sim(s, integrator="rk4", adaptive=False, dt=0.5 * rg.ic.K, precision="fp64_exact",
                stage_exact=True) as sim:
        assert sim.info(0).active == 0
        sim.step()
        info = sim.info(0)
        out = sim.get_state(0)
    assert info.t == 0.0 and info.n_tried == 0
    assert out.r.tobytes() == s.r.tobytes() and out.v.tobytes() == s.v.tobytes()


@pytest.mark.parametrize("shape", [dict(n_pp=1, n_pl=0), dict(n_pp=0, n_pl=300), dict(n_pp=0, n_pl=0, n_tp=40),
                                   dict(n_pp=2, n_pl=1)])
def test_degenerate_systems_bitexact(rg, orc, shape):
    s = disk(rg, **shape)
    out, b = fixed_run(rg, orc, s)
    assert np.array_equal(vec(out.r), vec(b.r))
    assert np.array_equal(vec(out.v), vec(b.v))


@pytest.mark.parametrize("precision", ["fp64_exact", "mixed"])
def test_inactive_bodies_are_skipped(rg, orc, precision):
    s = disk(rg, n_pp=4, n_pl=400, n_tp=5, seed=9)
    for k in (2, 7, 150, 401):   # a protoplanet, planetesimals, a test particle
        s.md["id"][k] *= -1
    kw = dict(integrator="rk4", adaptive=False, dt=0.01, precision=precision)
    if precision == "fp64_exact":
        kw["stage_exact"] = True
    with rg.Sim(s, **kw) as sim:
        a = vec(sim.calc_dydx(0, 1, 0.0))
    _, ref = orc.grav_accel(obody(orc, s), sem=orc.SEM_GPU)
    ref = vec(ref)
    live = s.md["id"] > 0
    assert np.all(a[~live] == 0.0)          # calc_grav_accel_naive zeroes inactive sinks
    if precision == "fp64_exact":
        assert np.array_equal(a, ref)
    else:
        err = np.linalg.norm(a[live] - ref[live], axis=1) / np.linalg.norm(ref[live], axis=1)
        assert err[0] < 2e-6 and err[1:].max() < 1e-9


def ragged(rg):
    """A lone star, a two-body system, a disk without protoplanets, a test-particle
    swarm and a disk large enough for chunked source lists."""
    return [disk(rg, n_pp=0, n_pl=0), disk(rg, n_pp=1, n_pl=0, seed=4), disk(rg, n_pp=0, n_pl=257, seed=5),
            disk(rg, n_pp=0, n_pl=0, n_tp=33, seed=6), disk(rg, n_pp=6, n_pl=2500, seed=7)]


def run_alone_and_together(rg, systems, kw, steps):
    singles = []
    for s in systems:
        with rg.Sim(s, **kw) as sim:
            for _ in range(steps):
                sim.step()
            singles.append((sim.get_state(0), sim.info(0)))
    together = []
    with rg.Sim(systems, **kw) as sim:
        for _ in range(steps):
            sim.step()
        for k in range(len(systems)):
            together.append((sim.get_state(k), sim.info(k)))
    return singles, together


def test_ragged_ensemble_equals_single_systems(rg):
    """FP64_EXACT, adaptive RKF7(8): every system of the ensemble ends bit for
    bit where it ends alone (same t, same tries)."""
    kw = dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K, precision="fp64_exact",
              stage_exact=True)
    singles, together = run_alone_and_together(rg, ragged(rg), kw, 4)
    for k, ((st1, i1), (st, i)) in enumerate(zip(singles, together)):
        assert i.t == i1.t and i.n_tried == i1.n_tried, k
        assert np.array_equal(vec(st.r), vec(st1.r)), k
        assert np.array_equal(vec(st.v), vec(st1.v)), k


@pytest.mark.parametrize("cluster", ["1", "0"])
def test_ragged_ensemble_mixed(rg, monkeypatch, cluster):
    """MIXED, RK4 fixed step, cluster plan on or off: the ensemble's launch plan
    chunks the large disk differently from its single-system plan (chunk sizes
    follow the whole launch), so the FP32 sums round differently; positions agree
    to 1e-12 relative after 4 steps."""
    monkeypatch.setenv("REDGB_CLUSTER", cluster)
    kw = dict(integrator="rk4", adaptive=False, dt=0.5 * rg.ic.K, precision="mixed")
    singles, together = run_alone_and_together(rg, ragged(rg), kw, 4)
    for k, ((st1, i1), (st, i)) in enumerate(zip(singles, together)):
        assert i.t == i1.t, k
        a, b = vec(st.r), vec(st1.r)
        scale = np.linalg.norm(b, axis=1).max() if len(b) > 1 else 1.0
        assert np.abs(a - b).max() <= 1e-12 * max(scale, 1e-300), k


def test_persistent_ensemble_equals_single_systems(rg):
    """An ensemble of more work items than one wave of CTAs holds (48 disks,
    ~1500 items) runs the per-variant stage instances (7 CTAs per SM); alone,
    each disk runs the one-wave instance that takes the variant as an argument.
    FP64_EXACT, adaptive RKF7(8) through red_step (step quotas leave systems idle
    for some tries): every disk ends bit for bit where it ends alone."""
    rng = np.random.Generator(np.random.MT19937(21))
    systems = [disk(rg, n_pp=int(rng.integers(0, 6)), n_pl=int(rng.integers(600, 1400)), seed=100 + k)
               for k in range(48)]
    systems[5] = disk(rg, n_pp=0, n_pl=0)   # a lone star: finished from the start
    assert sum(s.n // 32 for s in systems) > 6 * 152
    kw = dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K, precision="fp64_exact",
              stage_exact=True)
    singles, together = run_alone_and_together(rg, systems, kw, 3)
    for k, ((st1, i1), (st, i)) in enumerate(zip(singles, together)):
        assert i.t == i1.t and i.n_tried == i1.n_tried, k
        assert np.array_equal(vec(st.r), vec(st1.r)), k
        assert np.array_equal(vec(st.v), vec(st1.v)), k


def concat(states):
    # dtype= keeps red's record layout (a plain concatenate packs the metadata's padding away)
    return {f: np.concatenate([getattr(st, f) for st in states], dtype=getattr(states[0], f).dtype)
            for f in ("r", "v", "p", "md")}


class Records:
    def __init__(self, d):
        self.r, self.v, self.p, self.md = d["r"], d["v"], d["p"], d["md"]


def pinned_records(d):
    torch = pytest.importorskip("torch")
    out = {}
    for f, a in d.items():
        buf = torch.zeros(a.nbytes, dtype=torch.uint8).pin_memory()
        out[f] = buf.numpy().view(a.dtype)
        out[f][...] = a
        out[f + "_buf"] = buf
    return Records(out)


def same_records(a, b):
    for f in ("r", "v", "p"):
        assert getattr(a, f).tobytes() == getattr(b, f).tobytes(), f
    for f in a.md.dtype.names:
        assert np.array_equal(a.md[f], b.md[f]), f


def batched_setup(rg, holes):
    """A ragged ensemble; with holes, two disks whose collisions merge bodies
    and a compaction that shortens them (their device ranges then no longer
    follow each other)."""
    kw = dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K, precision="mixed")
    if not holes:
        return ragged(rg)[1:], kw, lambda sim: None
    from test_gpu_parity import collide_disk
    systems = [collide_disk(rg), disk(rg, n_pp=2, n_pl=150, seed=8), collide_disk(rg), disk(rg, n_pp=1, n_pl=90)]
    kw = dict(integrator="rk4", adaptive=False, dt=0.5 * rg.ic.K, precision="mixed", collision_factor=1.0)

    def merge(sim):
        sim.launch_tries(1)
        sim.synchronize()
        sim.handle_events()
        sim.rebuild_vectors()
    return systems, kw, merge


@pytest.mark.parametrize("holes", [False, True])
def test_batched_state_calls(rg, holes):
    """red_get_states / red_set_states over an ensemble equal the per-system
    calls, into pageable and pinned arrays; with holes the calls go system by
    system."""
    systems, kw, prepare = batched_setup(rg, holes)
    fields = ("r", "v", "p", "md")
    with rg.Sim(systems, **kw) as sim:
        prepare(sim)
        if holes:
            assert sim.info(0).n_total < systems[0].n and sim.info(2).n_total < systems[2].n
        sim.step()
        n = sim.bodies()
        per = Records(concat([sim.get_state(k) for k in range(sim.n_systems)]))
        assert len(per.r) == n
        same_records(per, sim.get_states(Records({f: np.zeros_like(getattr(per, f)) for f in fields})))
        same_records(per, sim.get_states(pinned_records({f: np.zeros_like(getattr(per, f)) for f in fields})))
        lo, m = sim.bodies(0, 1), sim.bodies(1, 2)
        part = sim.get_states(Records({f: np.zeros_like(getattr(per, f)[:m]) for f in fields}), sys0=1, count=2)
        same_records(Records({f: getattr(per, f)[lo:lo + m] for f in fields}), part)
        moved = Records({f: getattr(per, f).copy() for f in fields})
        moved.r["x"] += 1e-9
        moved.v["z"] *= 1.0 + 1e-9
    ends = []
    for how in ("per-system", "batched", "batched-pinned"):
        with rg.Sim(systems, **kw) as sim:
            prepare(sim)
            sim.step()
            if how == "per-system":
                a = 0
                for k in range(sim.n_systems):
                    m = sim.bodies(k, 1)
                    sim.set_state(k, Records({f: getattr(moved, f)[a:a + m] for f in fields}), parts="rv")
                    a += m
            elif how == "batched":
                sim.set_states(moved, parts="rv")
            else:
                sim.set_states(pinned_records({f: getattr(moved, f) for f in fields}), parts="rv")
            sim.step()
            ends.append(sim.get_states(Records({f: np.zeros_like(getattr(per, f)) for f in fields})))
    same_records(ends[0], ends[1])
    same_records(ends[0], ends[2])
