"""Synthetic planetesimal disks built with red's IC generator's random source
and recipe.

Follows src/red.cuda.initial: red_random and its distributions
(distribution.cpp:11-204; every drawn quantity has its own MT19937 stream,
seeded I[0] = seed), populate_disk (main.cu:251-314), calculate_phase
(main.cu:317-342) with tools::calc_phase and kepler_equation_solver
(tools.cpp:715-828: mu = K^2 (m_0 + m), red's solver and its tolerance),
then transform_to_bc (tools.cpp:384-434) and velocities divided by k so that
time is in red's code unit 1/k day (main.cu:2786-2790).  The disks' layouts
(protoplanets at given semi-major axes, mass weights) are this project's
workload definitions.

Units: AU, M_sun, code time (1/k day).
"""
import math

import numpy as np

from .types import (BMD, PARAM, PLANETESIMAL, PROTOPLANET, STAR, SUPERPLANETESIMAL, TESTPARTICLE,
                    VAR4, System)

K = 0.01720209895                       # red_macro.h:13
K2 = 0.0002959122082855911025           # red_macro.h:14
SOLAR_TO_EARTH = 3.3294605e5            # red_constants.h:132
EARTH_TO_SOLAR = 1.0 / SOLAR_TO_EARTH
AU_TO_METER = 1.495978707e11            # red_constants.h:162
AU_TO_CM = AU_TO_METER * 1.0e2
AU_TO_KM = AU_TO_METER / 1.0e3
SOLAR_RADIUS_TO_AU = 1.0 / 215.094      # red_constants.h:165,169
SOLAR_TO_GRAM = 1.0e3 * 1.98911e30      # red_constants.h:142-143
GRAM_TO_SOLAR = 1.0 / SOLAR_TO_GRAM
METER_TO_AU = 1.0 / AU_TO_METER          # red_constants.h:167
_CM_AU = 1.0e-2 * METER_TO_AU
G_CM3_TO_SOLAR_AU3 = GRAM_TO_SOLAR / (_CM_AU * _CM_AU * _CM_AU)   # red_constants.h:184
YEAR_TO_DAY = 365.25
FOUR_PI_OVER_THREE = 4.188790204786391  # tools.cpp:457
PI = 3.1415926535897932384626           # red_macro.h:16


class RedStreams:
    """red's random source for one disk: the k-th quantity drawn gets its own
    red_random stream (MT19937 seeded I[0] = seed, distribution.cpp:11-20,
    the stream of numpy's MT19937 under its legacy integer seeding), seeded
    64 seed + k, as red gives every distribution object its own seed.  The
    formulas are red's: uniform(a, b) = a + (b - a)(rand() + 1) / 2^32
    (distribution.cpp:36-44), Rayleigh sigma sqrt(-2 ln u) (:105-109), the
    power law by rejection (:141-162) and integers by red_random::uniform(int)
    (:46-49)."""

    def __init__(self, seed):
        self.seed = int(seed)
        self.k = 0

    def _raw(self, n):
        bg = np.random.MT19937(0)
        bg._legacy_seeding((64 * self.seed + self.k) & 0xFFFFFFFF)
        self.k += 1
        return bg.random_raw(n).astype(np.float64)

    def uniform(self, lo, hi, n):
        return lo + (hi - lo) * (self._raw(n) + 1.0) / 4294967296.0

    def rayleigh(self, sigma, n):
        u = (self._raw(n) + 1.0) / 4294967296.0
        return np.fromiter((sigma * math.sqrt(-2.0 * math.log(x)) for x in u), float, n)

    def power(self, lo, hi, power, n):
        """power_law_distribution::get_next, n times: every attempt takes two
        consecutive draws (x, then y), so the accepted values are the first n
        accepted pairs of the stream."""
        y_min = 0.0 if power == 0.0 else math.pow(lo, power)
        y_max = 1.0 if power == 0.0 else math.pow(hi, power)
        y_min, y_max = min(y_min, y_max), max(y_min, y_max)
        d_y, d_x = y_max - y_min, hi - lo
        area = d_x * d_y
        bg = np.random.MT19937(0)
        bg._legacy_seeding((64 * self.seed + self.k) & 0xFFFFFFFF)
        self.k += 1
        out = []
        while len(out) < n:
            raw = bg.random_raw(2 * max(1024, 4 * (n - len(out)))).astype(np.float64).reshape(-1, 2)
            x = (0.0 + (area - 0.0) * (raw[:, 0] + 1.0) / 4294967296.0) / d_y + lo
            y = y_min + (y_max - y_min) * (raw[:, 1] + 1.0) / 4294967296.0
            ok = np.fromiter((not (yy > math.pow(xx, power)) for xx, yy in zip(x, y)), bool, len(x))
            out.extend(x[ok][:n - len(out)])
        return np.array(out[:n])

    def integer(self, lo, hi):
        """red_random::uniform(int x_min, int x_max): one value in [lo, hi]."""
        r = self._raw(1)[0]
        return lo + int(r / 4294967296. * (hi - lo + 1))


def calc_radius(m, density):
    """tools::calc_radius, tools.cpp:455-460."""
    return np.power(1.0 / FOUR_PI_OVER_THREE * m / density, 1.0 / 3.0)


def calc_density(m, R):
    """tools::calc_density, tools.cpp:462-472."""
    R = np.asarray(R, dtype=float)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(R == 0.0, 0.0, m / (FOUR_PI_OVER_THREE * R ** 3))


def kepler_E(ecc, mean):
    """tools::kepler_equation_solver as calc_phase calls it (tools.cpp:715-755,
    789-795; tolerance 1e-8, at most 34 Newton steps from red's starting
    value), vectorised.  For a mean anomaly above pi red's solver ends with
    E = (mean - pi) + pi -- the mean anomaly itself, not the solution -- and
    so does this one, so that the disks are the ones red's generator makes."""
    ecc = np.asarray(ecc, float)
    mean = np.asarray(mean, float)
    trivial = (ecc == 0.0) | (mean == 0.0) | (mean == PI)
    upper = mean > PI
    m = np.where(upper, mean - PI, mean)
    E = m + ecc * np.sin(m) / (1.0 - np.sin(m + ecc) + np.sin(m))
    settled = np.zeros(E.shape, bool)
    for _ in range(34):
        step = E - (E - ecc * np.sin(E) - m) / (1.0 - ecc * np.cos(E))
        moved = np.abs(step - E)
        E = np.where(settled, E, step)
        settled |= moved <= 1.0e-8
        if settled.all():
            break
    E = np.where(upper, E + ((m - E) + PI), E)
    return np.where(trivial, mean, E)


def calc_phase(mu, a, e, inc, peri, node, mean):
    """tools::calc_phase, tools.cpp:789-828 (vectorised).  Returns r, v (n x 3)."""
    E = kepler_E(e, mean)
    nu = 2.0 * np.arctan(np.sqrt((1.0 + e) / (1.0 - e)) * np.tan(E / 2.0))
    p = a * (1.0 - e * e)
    r = p / (1.0 + e * np.cos(nu))
    ksi, eta = r * np.cos(nu), r * np.sin(nu)
    vk = -np.sqrt(mu / p) * np.sin(nu)
    ve = np.sqrt(mu / p) * (e + np.cos(nu))
    cw, sw, cO, sO, ci, si = np.cos(peri), np.sin(peri), np.cos(node), np.sin(node), np.cos(inc), np.sin(inc)
    P = np.stack([cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si], axis=1)
    Q = np.stack([-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si], axis=1)
    rv = np.stack([ksi * P[:, c] + eta * Q[:, c] for c in range(3)], axis=1)
    vv = np.stack([vk * P[:, c] + ve * Q[:, c] for c in range(3)], axis=1)
    return rv, vv


def to_barycentre(mass, r, v):
    """tools::transform_to_bc (tools.cpp:384-434): total mass and moments summed
    from the last body to the first (sequential sums, as red's loop), then
    subtracted; r and v are structured var4 arrays, updated in place."""
    M = np.cumsum(mass[::-1])[-1]
    for c in "xyz":
        r[c] -= np.cumsum((mass * r[c])[::-1])[-1] / M
        v[c] -= np.cumsum((mass * v[c])[::-1])[-1] / M


def hill_spaced(a0, n, m, m_star, k_hill=10.0):
    """Semi-major axes of n equal-mass bodies spaced k_hill mutual Hill radii apart."""
    h = ((2.0 * m) / (3.0 * m_star)) ** (1.0 / 3.0)
    f = (1.0 + 0.5 * k_hill * h) / (1.0 - 0.5 * k_hill * h)
    return a0 * f ** np.arange(n)


def build_system(rng, *, m_star=1.0, pp_a, pp_mass, pl_a, pl_mass, pl_radius=None,
                 sigma_e_pp=0.01, sigma_i_pp=0.005, sigma_e=0.01, sigma_i=0.005,
                 density_gcm3=2.0, cd=0.0, n_tp=0, pl_type=PLANETESIMAL, star_radius=None):
    """One disk: star + protoplanets + planetesimals (+ test particles), bodies
    sorted by type as red requires.  Masses in M_sun, a in AU."""
    n_pp, n_pl = len(pp_a), len(pl_a)
    n = 1 + n_pp + n_pl + n_tp
    rho = density_gcm3 * G_CM3_TO_SOLAR_AU3
    a = np.concatenate([pp_a, pl_a, rng.uniform(0.7, 1.5, n_tp)])
    m = np.concatenate([np.full(n_pp, pp_mass), np.asarray(pl_mass, float) * np.ones(n_pl), np.zeros(n_tp)])
    nb = n - 1
    e = np.abs(np.concatenate([rng.rayleigh(sigma_e_pp, n_pp), rng.rayleigh(sigma_e, n_pl + n_tp)]))
    e = np.minimum(e, 0.9)
    inc = np.abs(np.concatenate([rng.rayleigh(sigma_i_pp, n_pp), rng.rayleigh(sigma_i, n_pl + n_tp)]))
    peri, node, mean = (rng.uniform(0.0, 2.0 * PI, nb) for _ in range(3))
    mu = K2 * (m_star + m)
    rv, vv = calc_phase(mu, a, e, inc, peri, node, mean)       # AU, AU/day

    r = np.zeros(n, VAR4)
    v = np.zeros(n, VAR4)
    p = np.zeros(n, PARAM)
    md = np.zeros(n, BMD)
    r["x"][1:], r["y"][1:], r["z"][1:] = rv[:, 0], rv[:, 1], rv[:, 2]
    v["x"][1:], v["y"][1:], v["z"][1:] = vv[:, 0], vv[:, 1], vv[:, 2]
    p["mass"][0] = m_star
    p["radius"][0] = SOLAR_RADIUS_TO_AU if star_radius is None else star_radius
    p["density"][0] = calc_density(m_star, p["radius"][0])
    p["mass"][1:] = m
    p["density"][1:1 + n_pp + n_pl] = rho
    if pl_radius is not None:
        p["radius"][1 + n_pp:1 + n_pp + n_pl] = pl_radius
        p["mass"][1 + n_pp:1 + n_pp + n_pl] = FOUR_PI_OVER_THREE * np.asarray(pl_radius) ** 3 * rho
        p["radius"][1:1 + n_pp] = calc_radius(p["mass"][1:1 + n_pp], rho)
    else:
        p["radius"][1:1 + n_pp + n_pl] = calc_radius(p["mass"][1:1 + n_pp + n_pl], rho)
    p["cd"][1 + n_pp:1 + n_pp + n_pl] = cd
    md["id"] = np.arange(1, n + 1)
    md["body_type"][0] = STAR
    md["body_type"][1:1 + n_pp] = PROTOPLANET
    md["body_type"][1 + n_pp:1 + n_pp + n_pl] = pl_type
    md["body_type"][1 + n_pp + n_pl:] = TESTPARTICLE

    to_barycentre(p["mass"], r, v)
    # velocities in AU per code time unit (1/k day)
    for c in "xyz":
        v[c] /= K
    playing = np.zeros(7, np.uint32)
    playing[STAR] = 1
    playing[PROTOPLANET] = n_pp
    playing[pl_type] = n_pl
    playing[TESTPARTICLE] = n_tp
    names = ["star"] + ["pp%d" % i for i in range(n_pp)] + ["pl%d" % i for i in range(n_pl)] + \
            ["tp%d" % i for i in range(n_tp)]
    return System(r, v, p, md, playing, names)


def config1(seed=1, n_pl=2048):
    """Star 1 M_sun, 4 protoplanets of 0.1 M_earth at 0.8-1.4 AU, n_pl equal-mass
    planetesimals (1 M_earth in total), a ~ U[0.7, 1.5], sigma_e 0.01, sigma_i 0.005."""
    rng = RedStreams(seed)
    pl_a = rng.uniform(0.7, 1.5, n_pl)
    return build_system(rng, pp_a=np.array([0.8, 1.0, 1.2, 1.4]), pp_mass=0.1 * EARTH_TO_SOLAR,
                        pl_a=pl_a, pl_mass=EARTH_TO_SOLAR / n_pl)


def config2(seed=2, n_pp=16, n_pl=16367):
    """16 protoplanets of 0.05 M_earth spaced 10 mutual Hill radii from 0.5 AU;
    planetesimals log-uniform in [0.5, 3] AU with m ~ a^0.5 (surface density
    ~ r^-1.5), 1 M_earth in total; sigma_e 0.02, sigma_i 0.01."""
    rng = RedStreams(seed)
    mpp = 0.05 * EARTH_TO_SOLAR
    pl_a = rng.power(0.5, 3.0, -1.0, n_pl)   # log-uniform: red's power law with power -1
    w = pl_a ** 0.5
    pl_m = EARTH_TO_SOLAR * w / w.sum()
    return build_system(rng, pp_a=hill_spaced(0.5, n_pp, mpp, 1.0), pp_mass=mpp, pl_a=pl_a, pl_mass=pl_m,
                        sigma_e_pp=0.02, sigma_i_pp=0.01, sigma_e=0.02, sigma_i=0.01)


def config3(seed=3, n_pp=32, n_pl=65503):
    """32 protoplanets (0.05 M_earth, 10 mutual Hill radii from 0.5 AU) and
    planetesimals with a in [0.5, 4] AU and radii log-uniform in 1-100 km at
    2 g/cm^3, C_D = 0.44 (gas drag run)."""
    rng = RedStreams(seed)
    mpp = 0.05 * EARTH_TO_SOLAR
    pl_a = rng.uniform(0.5, 4.0, n_pl)
    R = rng.power(1.0, 100.0, -1.0, n_pl) / AU_TO_KM   # log-uniform radii
    return build_system(rng, pp_a=hill_spaced(0.5, n_pp, mpp, 1.0), pp_mass=mpp, pl_a=pl_a, pl_mass=0.0,
                        pl_radius=R, sigma_e_pp=0.01, sigma_i_pp=0.005, sigma_e=0.01, sigma_i=0.005,
                        cd=0.44)


def config4_system(i, n_min=128, n_max=4096):
    """System i of the ensemble: built like config 1 with its own seed
    (1000 + i), N ~ U[n_min, n_max] and 2-8 protoplanets."""
    rng = RedStreams(1000 + i)
    n = rng.integer(n_min, n_max)
    n_pp = rng.integer(2, 8)
    n_pl = n - 1 - n_pp
    pp_a = 0.8 + 0.2 * np.arange(n_pp)
    pl_a = rng.uniform(0.7, 1.5, n_pl)
    return build_system(rng, pp_a=pp_a, pp_mass=0.1 * EARTH_TO_SOLAR, pl_a=pl_a,
                        pl_mass=EARTH_TO_SOLAR / n_pl)


def config4(n_systems=512, n_min=128, n_max=4096, first=0):
    """Systems first .. first + n_systems - 1 of the ensemble."""
    return [config4_system(first + i, n_min, n_max) for i in range(n_systems)]


def config4_specs(n_systems=512, n_min=128, n_max=4096, first=0):
    """red_populate_disks specifications of the config-4 ensemble: the same
    system sizes as config4 (drawn from the same seeds), the bodies drawn on
    the GPU from Philox streams keyed by 1000 + i (a different realisation of
    the same recipe)."""
    from .lib import DiskSpec
    out = []
    for i in range(first, first + n_systems):
        rng = RedStreams(1000 + i)
        n = rng.integer(n_min, n_max)
        n_pp = rng.integer(2, 8)
        n_pl = n - 1 - n_pp
        out.append(DiskSpec(n_pp=n_pp, n_pl=n_pl, m_star=1.0, star_radius=SOLAR_RADIUS_TO_AU,
                            pp_mass=0.1 * EARTH_TO_SOLAR, pp_a0=0.8, pp_da=0.2, pp_hill=0.0, pl_a_min=0.7,
                            pl_a_max=1.5, pl_a_log=0, pl_mass_total=EARTH_TO_SOLAR, pl_mass_exp=0.0,
                            sigma_e_pp=0.01, sigma_i_pp=0.005, sigma_e=0.01, sigma_i=0.005, e_max=0.9,
                            density=2.0, cd=0.0, seed=1000 + i))
    return out


def config4_gpu(n_systems=512, n_min=128, n_max=4096, first=0, device=0):
    """The config-4 ensemble generated on the GPU (red_populate_disks)."""
    from .lib import populate_disks
    return populate_disks(config4_specs(n_systems, n_min, n_max, first), device=device)


def gas_disk_config3():
    """MMSN-like analytic gas disk of config 3 as red's analytic_gas_disk file
    keys (analytic_gas_disk.cu:99-246): Sigma_0 = 1700 g/cm^2, h/r = 0.05,
    eta = 0.002, rho_c = Sigma_0 / (sqrt(pi) h_0) because red's profile is
    exp(-(z/h)^2)."""
    h0_cm = 0.05 * AU_TO_CM
    rho_c = 1700.0 / (np.sqrt(np.pi) * h0_cm)
    return {"name": "mmsn", "time_dependence": "constant", "eta_c": 0.002, "eta_p": 0.0,
            "rho_c": rho_c, "rho_p": -2.5, "sch_c": 0.05, "sch_p": 1.0,
            "mmw": 2.3, "diameter": 3.0e-10, "alpha": 2.0e-3, "tau_c": 0.0, "tau_p": 0.0}


def write_gas_file(path, keys):
    with open(path, "w") as f:
        for k, v in keys.items():
            f.write("%s = %s\n" % (k, v if isinstance(v, str) else repr(float(v))))


def gas_params(keys, m_star=1.0):
    """analytic_gas_disk::set_param + calc + transform_time
    (analytic_gas_disk.cu:90-291) -> analytic_gas_disk_params_t record."""
    from .types import GAS
    gram_to_solar = GRAM_TO_SOLAR
    g = np.zeros(1, GAS)[0]
    dec = {"constant": 0, "const": 0, "linear": 1, "lin": 1, "exponential": 2, "exp": 2}
    g["gas_decrease"] = dec[keys.get("time_dependence", "constant")]
    kk = K
    g["t0"] = float(keys.get("t0", 0.0)) * YEAR_TO_DAY * kk
    g["t1"] = float(keys.get("t1", 0.0)) * YEAR_TO_DAY * kk
    g["e_folding_time"] = float(keys.get("e_folding_time", 0.0)) * YEAR_TO_DAY * kk
    g["alpha"] = float(keys.get("alpha", 0.0))
    g["mean_molecular_weight"] = float(keys.get("mmw", 0.0)) * gram_to_solar
    g["particle_diameter"] = float(keys.get("diameter", 0.0)) * METER_TO_AU
    g["eta"] = (float(keys.get("eta_c", 0.0)), float(keys.get("eta_p", 0.0)))
    g["rho"] = (float(keys.get("rho_c", 0.0)) * G_CM3_TO_SOLAR_AU3, float(keys.get("rho_p", 0.0)))
    g["sch"] = (float(keys.get("sch_c", 0.0)), float(keys.get("sch_p", 0.0)))
    g["tau"] = (float(keys.get("tau_c", 0.0)), float(keys.get("tau_p", 0.0)))
    return g


def benchmark_cube(n, seed=0):
    """red's benchmark workload: n unit-mass bodies uniform in [-50, 50]^3
    (red.cuda.benchmark/main.cu:1793-1804), all of type protoplanet (SI) so
    every pair interacts."""
    rng = np.random.Generator(np.random.MT19937(seed))
    r = np.zeros(n, VAR4)
    v = np.zeros(n, VAR4)
    p = np.zeros(n, PARAM)
    md = np.zeros(n, BMD)
    for c in "xyz":
        r[c] = rng.uniform(-50.0, 50.0, n)
    p["mass"] = 1.0
    p["radius"] = 1e-3
    p["density"] = 1.0
    md["id"] = np.arange(1, n + 1)
    md["body_type"] = PROTOPLANET
    playing = np.zeros(7, np.uint32)
    playing[PROTOPLANET] = n
    return System(r, v, p, md, playing, ["b%d" % i for i in range(n)])
