"""The bench's workloads at their full sizes, checked through size-independent
properties (the oracle would take minutes at these sizes).

* the 16384-body disk (MIXED, adaptive RKF7(8) at tol 1e-10; collisions off, since a
  perfect merge changes E by design): energy over the interacting pairs
  conserved to |dE/E| < 1e-9 and the angular momentum to 1e-10 over 300 tries,
  the metric's accuracy bar.
* the 512-disk ensemble (1.08 M bodies): the same bar for every disk after 30 tries,
  and the ensemble's counters consistent (tried = passed + failed).
* the same disk with every pair interacting: the same bar after 8 tries.
* the 2053-body disk (RK4 fixed step): MIXED against FP64 after 100 steps, 1e-10
  relative in position (the precision modes agree at full size).
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
