"""CPU restatement of red_populate_disks (test infrastructure: the checker of
the GPU disk generator, never called by the library).

The generator follows red.cuda.initial's disk recipe (populate_disk,
red.cuda.initial/main.cu:251-314; calculate_phase, main.cu:317-342;
distribution.cpp:105-109 for the Rayleigh draws; tools.cpp:413-434, 455-472,
716-749, 789-828 for the barycentre, radius / density, Kepler solver and
Kepler -> Cartesian; the Kepler solver is oracle/red_initial.py's, pinned to
red's compiled generator), with Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel
random numbers: as easy as 1, 2, 3", SC'11) as the random source: key = the
system's seed, counter = (body, draw block, 0, 0).  The integer stream is
exact; the floating-point math uses numpy's libm, so results agree with the
GPU's to rounding of the math functions (about 1e-15 relative).
"""
import numpy as np

from .red_initial import kepler_E   # red's solver, pinned to red.cuda.initial

K = 0.01720209895
K2 = 0.0002959122082855911025
FOUR_PI_OVER_THREE = 4.188790204786391
TWO_PI = 6.283185307179586
_CM_AU = 1.0e-2 / 1.495978707e11
RHO_UNIT = (1.0 / (1.0e3 * 1.98911e30)) / (_CM_AU * _CM_AU * _CM_AU)

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: (n, 4) uint32, key: (2,) ints.  Returns the (n, 4) uint32 output."""
    c = [np.asarray(ctr[:, q], np.uint64) for q in range(4)]
    k0, k1 = int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ np.uint64(k0), lo1, hi0 ^ c[3] ^ np.uint64(k1), lo0]
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return np.stack([x.astype(np.uint32) for x in c], axis=1)


def u01(hi, lo):
    b = ((hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)) >> np.uint64(11)
    return (b + np.uint64(1)).astype(np.float64) * 1.1102230246251565e-16


def draws(seed, n):
    """The six draws of bodies 1 .. n - 1 (rows), columns u0 .. u5."""
    k = np.arange(1, n, dtype=np.uint32)
    key = (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    u = np.zeros((n - 1, 6))
    for b in range(3):
        ctr = np.zeros((n - 1, 4), np.uint32)
        ctr[:, 0] = k
        ctr[:, 1] = b
        out = philox4x32_10(ctr, key)
        u[:, 2 * b] = u01(out[:, 0], out[:, 1])
        u[:, 2 * b + 1] = u01(out[:, 2], out[:, 3])
    return u


def populate(spec):
    """One disk from a dict with the fields of red_disk_spec_t: (r, v, mass,
    radius, density, cd, id, body_type) as arrays, r and v (n, 3)."""
    n_pp, n_pl = int(spec["n_pp"]), int(spec["n_pl"])
    n = 1 + n_pp + n_pl
    u = draws(int(spec["seed"]), n)
    j = np.arange(n_pp)
    if spec["pp_hill"] > 0.0:
        h = np.cbrt(2.0 * spec["pp_mass"] / (3.0 * spec["m_star"]))
        f = (1.0 + 0.5 * spec["pp_hill"] * h) / (1.0 - 0.5 * spec["pp_hill"] * h)
        a_pp = spec["pp_a0"] * np.power(f, j.astype(float))
    else:
        a_pp = spec["pp_a0"] + j * spec["pp_da"]
    up = u[n_pp:, 0]
    if spec["pl_a_log"]:
        lo, hi = np.log(spec["pl_a_min"]), np.log(spec["pl_a_max"])
        a_pl = np.exp(lo + up * (hi - lo))
    else:
        a_pl = spec["pl_a_min"] + up * (spec["pl_a_max"] - spec["pl_a_min"])
    a = np.concatenate([a_pp, a_pl])
    pp = np.arange(n - 1) < n_pp
    se = np.where(pp, spec["sigma_e_pp"], spec["sigma_e"])
    si = np.where(pp, spec["sigma_i_pp"], spec["sigma_i"])
    ecc = np.minimum(se * np.sqrt(-2.0 * np.log(u[:, 1])), spec["e_max"])
    inc = si * np.sqrt(-2.0 * np.log(u[:, 2]))
    peri, node, mean = TWO_PI * u[:, 3], TWO_PI * u[:, 4], TWO_PI * u[:, 5]
    w = np.power(a_pl, spec["pl_mass_exp"])
    m_pl = spec["pl_mass_total"] * w / (w.sum() if n_pl else 1.0)
    m = np.concatenate([np.full(n_pp, spec["pp_mass"]), m_pl])
    mu = K2 * (spec["m_star"] + m)
    E = kepler_E(ecc, mean)
    nu = 2.0 * np.arctan(np.sqrt((1.0 + ecc) / (1.0 - ecc)) * np.tan(0.5 * E))
    p = a * (1.0 - ecc * ecc)
    rr = p / (1.0 + ecc * np.cos(nu))
    ksi, eta = rr * np.cos(nu), rr * np.sin(nu)
    vk, ve = -np.sqrt(mu / p) * np.sin(nu), np.sqrt(mu / p) * (ecc + np.cos(nu))
    cw, sw, cO, sO, ci, sinc = np.cos(peri), np.sin(peri), np.cos(node), np.sin(node), np.cos(inc), np.sin(inc)
    P = np.stack([cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * sinc], axis=1)
    Q = np.stack([-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * sinc], axis=1)
    r = np.zeros((n, 3))
    v = np.zeros((n, 3))
    r[1:] = ksi[:, None] * P + eta[:, None] * Q
    v[1:] = vk[:, None] * P + ve[:, None] * Q
    mass = np.concatenate([[spec["m_star"]], m])
    rho = spec["density"] * RHO_UNIT
    radius = np.concatenate([[spec["star_radius"]], np.cbrt(m / (FOUR_PI_OVER_THREE * rho))])
    R = spec["star_radius"]
    density = np.concatenate([[spec["m_star"] / (FOUR_PI_OVER_THREE * R ** 3) if R else 0.0],
                              np.full(n - 1, rho)])
    cd = np.concatenate([[0.0], np.zeros(n_pp), np.full(n_pl, spec["cd"])])
    M = mass.sum()
    r -= (mass[:, None] * r).sum(axis=0) / M
    v -= (mass[:, None] * v).sum(axis=0) / M
    v /= K
    body_type = np.concatenate([[0], np.full(n_pp, 3), np.full(n_pl, 5)]).astype(np.int32)
    return {"r": r, "v": v, "mass": mass, "radius": radius, "density": density, "cd": cd,
            "id": np.arange(1, n + 1, dtype=np.int32), "body_type": body_type}
