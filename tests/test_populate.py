"""red_populate_disks: disk ensembles generated on the GPU.

The oracle (oracle/populate_oracle.py) restates the generator on the CPU with
the same Philox4x32-10 stream; the integer stream is exact, the floating-point
math goes through two different libms, so positions and velocities agree to
1e-12 relative, masses and radii to 1e-14, ids, types and counts exactly.
The Philox restatement itself is pinned on the known-answer vectors published
with the method (Random123 kat_vectors: counter / key 0; all ones; pi digits).
"""
import numpy as np
import pytest

from oracle import populate_oracle as po


def test_philox_known_answers():
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in cases:
        out = po.philox4x32_10(np.array([ctr], np.uint32), key)
        assert tuple(int(x) for x in out[0]) == want


def spec_dict(**kw):
    d = dict(n_pp=6, n_pl=3000, m_star=1.0, star_radius=1.0 / 215.094, pp_mass=0.1 / 3.3294605e5, pp_a0=0.8,
             pp_da=0.2, pp_hill=0.0, pl_a_min=0.7, pl_a_max=1.5, pl_a_log=0, pl_mass_total=1.0 / 3.3294605e5,
             pl_mass_exp=0.0, sigma_e_pp=0.01, sigma_i_pp=0.005, sigma_e=0.02, sigma_i=0.01, e_max=0.9,
             density=2.0, cd=0.0, seed=12345)
    d.update(kw)
    return d


def test_oracle_disk_statistics():
    d = po.populate(spec_dict(n_pl=20000))
    n_pp = 6
    r, v, m = d["r"], d["v"], d["mass"]
    assert np.abs((m[:, None] * r).sum(axis=0)).max() < 1e-16        # barycentric
    assert np.abs((m[:, None] * v).sum(axis=0)).max() < 1e-16
    pl = slice(1 + n_pp, None)
    rel = r[pl] - r[0]
    dist = np.linalg.norm(rel, axis=1)
    assert dist.min() > 0.7 * (1 - 0.2) and dist.max() < 1.5 * (1 + 0.2)
    # Rayleigh: mean sigma sqrt(pi / 2); i from z / r
    incl = np.arcsin(np.abs(rel[:, 2]) / dist)
    assert abs(np.abs(incl).mean() - 0.01 * np.sqrt(np.pi / 2) * 2 / np.pi) < 2e-3
    assert abs(m[pl].sum() - 1.0 / 3.3294605e5) < 1e-18
    assert list(d["body_type"][:8]) == [0, 3, 3, 3, 3, 3, 3, 5]


SPECS = [dict(), dict(pp_hill=10.0, pp_a0=0.5, n_pp=16, pl_a_min=0.5, pl_a_max=3.0, pl_a_log=1, pl_mass_exp=0.5,
                      seed=2), dict(n_pp=2, n_pl=129, cd=0.44, seed=7, sigma_e=0.05)]


@pytest.mark.gpu
def test_populate_matches_oracle(rg):
    specs = [rg.lib.DiskSpec(**spec_dict(**s)) for s in SPECS]
    systems = rg.lib.populate_disks(specs)
    for sp, s in zip(SPECS, systems):
        d = po.populate(spec_dict(**sp))
        n = len(d["mass"])
        assert s.n == n
        assert list(s.playing) == [1, 0, 0, spec_dict(**sp)["n_pp"], 0, spec_dict(**sp)["n_pl"], 0]
        assert np.array_equal(s.md["id"], d["id"]) and np.array_equal(s.md["body_type"], d["body_type"])
        for got, want in ((np.stack([s.r["x"], s.r["y"], s.r["z"]], axis=1), d["r"]),
                          (np.stack([s.v["x"], s.v["y"], s.v["z"]], axis=1), d["v"])):
            scale = np.linalg.norm(want, axis=1).max()
            assert np.abs(got - want).max() <= 1e-12 * scale
        for f in ("mass", "radius", "density", "cd"):
            assert np.allclose(s.p[f], d[f], rtol=1e-14, atol=0), f
        assert np.all(s.r["w"] == 0.0) and np.all(s.v["w"] == 0.0)


@pytest.mark.gpu
def test_populate_is_deterministic_and_seeded(rg):
    a = rg.lib.populate_disks([rg.lib.DiskSpec(**spec_dict(seed=5))])[0]
    b = rg.lib.populate_disks([rg.lib.DiskSpec(**spec_dict(seed=5))])[0]
    c = rg.lib.populate_disks([rg.lib.DiskSpec(**spec_dict(seed=6))])[0]
    assert a.r.tobytes() == b.r.tobytes() and a.v.tobytes() == b.v.tobytes()
    assert a.r.tobytes() != c.r.tobytes()


@pytest.mark.gpu
def test_populated_ensemble_integrates(rg):
    systems = rg.ic.config4_gpu(n_systems=8)
    with rg.Sim(systems, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * rg.ic.K,
                collision_factor=0.0) as sim:
        e0 = [sim.energy_interacting(k)[0] for k in range(len(systems))]
        sim.launch_tries(40)
        sim.synchronize()
        e1 = [sim.energy_interacting(k)[0] for k in range(len(systems))]
    for a, b in zip(e0, e1):
        assert abs((b - a) / a) < 1e-9


def test_populate_rejects_bad_specs(rg):
    bad = rg.lib.DiskSpec(**spec_dict(e_max=1.0))
    with pytest.raises(rg.RedError) as e:
        rg.lib.populate_disks([bad])
    assert e.value.code == 1   # RED_ERR_ARG, checked before any device call
