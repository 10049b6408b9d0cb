"""Pins the oracle (oracle/red_oracle.c) to the reference's own code.

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py,
which runs suliaron/red.cuda's CPU implementation (built unmodified from its
sources by oracle/ref_build.sh).  Integer and index results must be equal;
floating-point results must be bit-identical, since the oracle follows red's
expression order and is built without FMA contraction like red (-fmad=false).
"""
import numpy as np
import pytest

from conftest import golden


def body(orc, g):
    return orc.Body(g["r"], g["v"], g["p"], g["md"], g["playing"])


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8)


def test_grav_cpu_semantics_bitexact(orc):
    g = golden("grav_cpu_si.npz")
    b = body(orc, g)
    rc, a = orc.grav_accel(b, sem=orc.SEM_CPU)
    assert rc == 0 and int(g["ok"]) == 1
    assert np.array_equal(bits(a), bits(g["a"]))


def test_grav_gpu_semantics_close_to_cpu(orc):
    # red's GPU kernel sums sources in index order, its CPU path symmetrically:
    # same forces to rounding.
    g = golden("grav_cpu_si.npz")
    b = body(orc, g)
    rc, a = orc.grav_accel(b, sem=orc.SEM_GPU)
    assert rc == 0
    for c in "xyz":
        ref = g["a"][c]
        assert np.allclose(a[c], ref, rtol=1e-12, atol=1e-15 * np.abs(ref).max())


def test_cpu_semantics_refuse_planetesimals(orc, rg):
    s = rg.ic.config1(n_pl=16)
    b = orc.Body(s.r, s.v, s.p, s.md, s.playing)
    rc, _ = orc.grav_accel(b, sem=orc.SEM_CPU)
    assert rc == orc.ERR_NOT_IMPLEMENTED   # pp_disk.cu:974-982 throws


def test_drag_bitexact(orc):
    g = golden("drag.npz")
    b = body(orc, g)
    a = np.zeros(b.n, orc.VAR4)
    gas = np.ascontiguousarray(g["gas"], dtype=orc.GAS)
    orc.lib().orc_drag_accel(float(g["t"]), orc._p(gas), *orc._u32(b.playing)[1:], orc._p(b.p),
                             orc._p(b.r), orc._p(b.v), orc._p(a))
    assert np.array_equal(bits(a), bits(g["a"]))
    nsi = int(b.playing[:4].sum())
    assert np.abs(a["x"][nsi:]).max() > 0.0 and np.all(a["x"][:nsi] == 0.0)


@pytest.mark.parametrize("name", ["rk4_fixed", "rk4_adaptive", "rkf78_adaptive",
                                  "rkf78_adaptive_tp", "rkf78_fixed", "euler_fixed", "rk2_fixed"])
def test_integrator_bitexact(orc, name):
    g = golden(name + ".npz")
    b = body(orc, g)
    kind = {1: orc.EULER, 2: orc.RK2, 4: orc.RK4, 8: orc.RKF78}[int(g["integrator"])]
    ig = orc.make_integrator(kind, float(g["dt0"]), adaptive=bool(g["adaptive"]), tol=float(g["tol"]),
                             error_check_for_tp=bool(g["eftp"]), sem=orc.SEM_CPU)
    t = 0.0
    for k, st in enumerate(g["steps"]):
        rc, t = orc.step(ig, b, t)
        assert rc == 0
        assert t == st["t"], k
        assert ig.dt_did == st["dt"], k
        assert ig.dt_next == st["dt_next"], k
        assert (ig.n_tried, ig.n_passed, ig.n_failed) == (st["tried"], st["passed"], st["failed"]), k
    assert np.array_equal(bits(b.r), bits(g["r_out"]))
    assert np.array_equal(bits(b.v), bits(g["v_out"]))
    I = orc.calc_integral(b)
    ref = g["integral"]   # pp_disk_t::integral_t: R(var4) V(var4) C(var4) E
    assert np.array_equal(I, np.concatenate([ref[0:3], ref[4:7], ref[8:11], ref[12:13]]))


def test_adaptive_runs_reject_some_steps(orc):
    g = golden("rkf78_adaptive.npz")
    assert g["steps"]["failed"][-1] >= 0
    assert g["steps"]["passed"][-1] == len(g["steps"])


def fields_equal(a, b, names):
    return all(np.array_equal(bits(np.ascontiguousarray(a[n])), bits(np.ascontiguousarray(b[n]))) for n in names)


def event_key_fields(ev):
    return [(int(e["event_name"]), int(e["id1"]), int(e["id2"]), int(e["idx1"]), int(e["idx2"])) for e in ev]


def test_collision_cpu_semantics_bitexact(orc):
    g = golden("collision_cpu.npz")
    b = body(orc, g)
    rc, ev, n = orc.check_collision(b, float(g["t"]), float(g["factor"]), sem=orc.SEM_CPU)
    assert rc == 0
    raw = g["raw"]
    assert n == len(raw) and n >= 4
    assert event_key_fields(ev) == event_key_fields(raw)
    assert fields_equal(ev, raw, ["t", "d", "r1", "v1", "r2", "v2", "r0", "v0", "p0"])
    rc, sp = orc.handle_collision(b, ev)
    assert rc == 0
    assert event_key_fields(sp) == event_key_fields(g["sp"])
    assert fields_equal(sp, g["sp"], ["p1", "p2", "ps", "rs", "vs"])
    assert np.array_equal(bits(b.r), bits(g["r_out"]))
    assert np.array_equal(bits(b.v), bits(g["v_out"]))
    assert np.array_equal(bits(b.p), bits(g["p_out"]))
    assert np.array_equal(b.md["id"], g["md_out"]["id"])
    assert np.array_equal(b.inactive, g["inactive"])


def test_collision_gpu_semantics_adds_star_pairs(orc):
    # red's GPU kernel does not skip the star as the first body (pp_disk.cu:336);
    # its CPU twin does (pp_disk.cu:1149).  The planted body inside the star shows it.
    g = golden("collision_cpu.npz")
    b = body(orc, g)
    _, ev_cpu, _ = orc.check_collision(b, 0.0, 1.0, sem=orc.SEM_CPU)
    _, ev_gpu, _ = orc.check_collision(b, 0.0, 1.0, sem=orc.SEM_GPU)
    cpu = set(event_key_fields(ev_cpu))
    gpu = set(event_key_fields(ev_gpu))
    assert cpu < gpu
    assert all(k[3] == 0 or k[4] == 0 for k in gpu - cpu)


def test_ejection_hit_centrum_and_rebuild_bitexact(orc):
    g = golden("ejhc.npz")
    b = body(orc, g)
    rc, ev, n = orc.check_ejection_hit_centrum(b, float(g["t"]), float(g["ej"]), float(g["hc"]))
    assert rc == 0
    assert event_key_fields(ev) == event_key_fields(g["raw"])
    assert fields_equal(ev, g["raw"], ["t", "d", "r1", "v1", "r2", "v2", "p1", "p2", "ps", "rs", "vs"])
    rc, ev2 = orc.handle_ejection_hit_centrum(b, ev)
    assert rc == 0
    assert np.array_equal(bits(b.r), bits(g["r_out"]))
    assert np.array_equal(bits(b.p), bits(g["p_out"]))
    assert np.array_equal(b.md["id"], g["md_out"]["id"])
    assert np.array_equal(b.inactive, g["inactive"])
    orc.rebuild_vectors(b)
    assert b.n == int(g["rb_n"])
    assert np.array_equal(b.playing, g["rb_playing"])
    assert np.array_equal(bits(b.r), bits(g["rb_r"]))
    assert np.array_equal(b.md["id"], g["rb_md"]["id"])


def test_integral_bitexact(orc):
    g = golden("integral.npz")
    b = body(orc, g)
    I = orc.calc_integral(b)
    ref = g["integral"]
    assert np.array_equal(I, np.concatenate([ref[0:3], ref[4:7], ref[8:11], ref[12:13]]))


# Known-answer tests of red's own unit tests (src/red.cuda.utility/red_test.cpp)
def test_kat_merge(orc):
    import ctypes as C
    V4 = orc.VAR4
    r1 = np.array([(1.0, 1.0, 1.0, 0.0)], V4); r2 = np.array([(4.0, 3.0, 1.0, 0.0)], V4)
    out = np.zeros(1, V4)
    orc.lib().orc_calc_position_after_collision(1.0, 1.0, orc._p(r1), orc._p(r2), orc._p(out))
    assert tuple(out[0])[:3] == (2.5, 2.0, 1.0)                      # red_test.cpp:798-830
    v1 = np.array([(1.0, 0.0, 0.0, 0.0)], V4); v2 = np.array([(-1.0, 0.0, 0.0, 0.0)], V4)
    orc.lib().orc_calc_velocity_after_collision(1.0, 1.0, orc._p(v1), orc._p(v2), orc._p(out))
    assert tuple(out[0])[:3] == (0.0, 0.0, 0.0)                      # red_test.cpp:833-860
    v1 = np.array([(-1.0, 0.0, 0.0, 0.0)], V4)
    orc.lib().orc_calc_velocity_after_collision(1.0, 1.0, orc._p(v1), orc._p(v1), orc._p(out))
    assert tuple(out[0])[:3] == (-1.0, 0.0, 0.0)                     # red_test.cpp:862-885
    p1 = np.array([(1.0, 1.0, 1.0, 1.0)], orc.PARAM)
    pr = np.zeros(1, orc.PARAM)
    orc.lib().orc_calc_physical_properties(orc._p(p1), orc._p(p1), orc._p(pr))
    assert pr["mass"][0] == 2.0 and pr["cd"][0] == 1.0               # red_test.cpp:886-930
    assert abs(pr["density"][0] - 0.23873241463784300365332564505877) < 1e-15
    assert pr["radius"][0] == orc.lib().orc_calc_radius(2.0, pr["density"][0])


def test_kat_barycentre(orc):
    # 4-body fixture create_sim_data (red_test.cpp:22-125); R0 = (0.5,0.5,0), V0 = (1.5,0,0)
    V4 = orc.VAR4
    r = np.array([(0, 0, 0, 0), (1, 0, 0, 0), (1, 1, 0, 0), (0, 1, 0, 0)], V4)
    v = np.array([(1, 0, 0, 0), (2, 0, 0, 0), (2, 0, 0, 0), (1, 0, 0, 0)], V4)
    p = np.array([(1.0, 1.0, 0.23873241463784300365332564505877, 0.0)] * 4, orc.PARAM)
    md = np.zeros(4, orc.BMD)
    md["id"] = [1, 1, 2, 3]
    md["body_type"] = [0, 1, 1, 3]
    b = orc.Body(r, v, p, md, [1, 2, 0, 1, 0, 0, 0])
    I = orc.calc_integral(b)
    assert np.allclose(I[0:3], [0.5, 0.5, 0.0], atol=1e-15)           # red_test.cpp:600-640
    assert np.allclose(I[3:6], [1.5, 0.0, 0.0], atol=1e-15)


def test_bounds(orc):
    # n_objects_t::get_bound_* (red_type.h:670-700), the cases of test.cu:7-449
    pl = [1, 2, 3, 4, 5, 6, 7]
    assert orc.bound(pl, 0) == (0, 10, 0, 21)
    assert orc.bound(pl, 1) == (10, 21, 0, 10)
    assert orc.bound(pl, 2) == (21, 28, 0, 21)
    assert orc.bound(pl, 3) == (10, 21, 0, 0)
    assert orc.interactions_per_eval([1, 0, 0, 16, 0, 16367, 0]) == 17 * 16383 + 16367 * 17


@pytest.mark.parametrize("name", ["initial_disk.npz", "initial_branches.npz"])
def test_initial_generator_matches_red(name):
    """oracle/red_initial.py against red.cuda.initial's own generator (golden
    vectors from oracle/_ref/initial_harness): every drawn and derived
    quantity bit for bit, positions and velocities to 1e-15 relative (numpy's
    sin / cos / atan / tan against the C library's)."""
    from oracle import red_initial
    g = golden(name)
    d, dt = red_initial.populate(bytes(g["spec"]).decode())
    assert np.array_equal(d["oe"], g["oe"])
    for f in ("mass", "radius", "density", "cd"):
        assert np.array_equal(d[f], g["p"][f]), f
    assert np.array_equal(d["id"], g["md"]["id"]) and np.array_equal(d["body_type"], g["md"]["body_type"])
    for q in ("r", "v"):
        ref = np.stack([g[q]["x"], g[q]["y"], g[q]["z"]], axis=1)
        assert np.allclose(d[q], ref, rtol=1e-15, atol=1e-15 * np.abs(ref).max()), q
    assert dt == pytest.approx(float(g["dt"]), rel=1e-15)


def test_ic_draws_and_recipe_follow_red(rg):
    """red.cuda_gb300/ic.py, the generator of the bench's disks, against the
    pinned restatement: its random source gives red's draws bit for bit, and
    its Kepler solver, element-to-Cartesian conversion and barycentre give the
    same state from the same elements (the golden disk's)."""
    from oracle import red_initial
    s = rg.ic.RedStreams(7)
    for k, (kind, args, n) in enumerate([("uniform", (0.7, 1.5), 500), ("rayleigh", (0.02,), 500),
                                         ("power", (0.5, 3.0, -1.0), 300)]):
        got = getattr(s, kind)(*args, n) if kind != "uniform" else s.uniform(*args, n)
        ref = red_initial.Distribution(kind, 64 * 7 + k, *args).draw(n)
        assert np.array_equal(got, ref), kind
    s = rg.ic.RedStreams(11)
    rr = red_initial.RedRandom(64 * 11)
    assert s.integer(128, 4096) == 128 + int(rr.rand() / 4294967296. * (4096 - 128 + 1))
    g = golden("initial_disk.npz")
    d, _ = red_initial.populate(bytes(g["spec"]).decode())
    oe, mass = d["oe"], d["mass"]
    mu = rg.ic.K2 * (mass[0] + mass[1:])
    r, v = rg.ic.calc_phase(mu, oe[1:, 0], oe[1:, 1], oe[1:, 2], oe[1:, 3], oe[1:, 4], oe[1:, 5])
    rr_, vv_ = red_initial.calc_phase(mu, oe[1:, 0], oe[1:, 1], oe[1:, 2], oe[1:, 3], oe[1:, 4], oe[1:, 5])
    assert np.array_equal(r, rr_) and np.array_equal(v, vv_)
    R = np.zeros(len(mass), rg.types.VAR4)
    V = np.zeros(len(mass), rg.types.VAR4)
    for k, c in enumerate("xyz"):
        R[c][1:], V[c][1:] = r[:, k], v[:, k]
    rg.ic.to_barycentre(mass, R, V)
    R2 = np.vstack([np.zeros(3), r])
    V2 = np.vstack([np.zeros(3), v])
    red_initial.transform_to_bc(mass, R2, V2, d["id"])
    for k, c in enumerate("xyz"):
        assert np.array_equal(R[c], R2[:, k]) and np.array_equal(V[c], V2[:, k])
