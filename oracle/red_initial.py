"""CPU restatement of red.cuda.initial's disk recipe -- TEST INFRASTRUCTURE.

Pinned against red's own generator (oracle/initial_harness.cu, built from
red's unmodified sources by oracle/ref_build.sh) through the golden vectors
tests/golden/initial_*.npz.  It is the checker of this project's two
generators: the numpy one the bench's workloads come from
(red.cuda_gb300/ic.py) and the GPU one (red_populate_disks, whose own
restatement, oracle/populate_oracle.py, takes its Kepler solver and
element-to-Cartesian conversion from here).

What red does, and this module restates:
* red_random (src/red.cuda.initial/distribution.cpp:11-46): MT19937 seeded by
  the 1812433253 recurrence from I[0] = seed; rand() is the tempered 32-bit
  output; uniform(a, b) = a + (b - a) (rand() + 1) / 2^32.  This is the
  stream of numpy's MT19937 bit generator under its legacy integer seeding
  (checked against red's compiled code).
* distributions (distribution.cpp:60-204): uniform, exponential, Rayleigh
  sigma sqrt(-2 ln u), normal, and the power law by rejection; every drawn
  quantity of every body type has its own distribution object and seed.
* populate_disk (main.cu:251-314): bodies in type order; per body the
  physical properties (mass, radius, density, drag coefficient, each drawn
  when its distribution exists) and then the orbital elements (sma, ecc,
  inc, peri, node, mean); the missing one of mass / radius / density from
  the other two; test particles massless; the primary star at rest at the
  origin.  generate_oe's retry loop never retries (its condition
  x_min > x && x_max < x cannot hold, util_init.cpp:56-65).
* the scenarios' fix-up of radius / density (main.cu:2764-2781),
  calculate_phase (main.cu:317-342) with tools::calc_phase and
  kepler_equation_solver (tools.cpp:715-755, 789-828: tolerance 1e-8; for a
  mean anomaly above pi the solver returns the mean anomaly itself, since
  `*E += (mean - *E) + PI` undoes its own solution), then transform_to_bc
  (tools.cpp:384-434, sums from the last body to the first), transform_time
  and transform_velocity (v / k).

Drawn quantities are bit-identical to red's.  Positions and velocities go
through sin, cos, atan, tan, sqrt and pow, evaluated here with numpy: they
agree with red's to ~1e-15 relative.
"""
import math

import numpy as np

K = 0.01720209895                  # red_macro.h:13
K2 = 0.0002959122082855911025      # red_macro.h:14
PI = 3.1415926535897932384626      # red_macro.h
FOUR_PI_OVER_THREE = 4.188790204786391
BODY_TYPE_N = 7
STAR, TESTPARTICLE, SUPERPLANETESIMAL = 0, 6, 4
PP_NAMES = ("mass", "radius", "density", "cd")
OE_NAMES = ("sma", "ecc", "inc", "peri", "node", "mean")


class RedRandom:
    """red_random: the raw MT19937 stream with red's seeding."""

    def __init__(self, seed):
        self.bg = np.random.MT19937(0)
        self.bg._legacy_seeding(int(seed) & 0xFFFFFFFF)

    def rand(self, n=None):
        if n is None:
            return int(self.bg.random_raw())
        return self.bg.random_raw(n).astype(np.float64)

    def uniform(self, n=None, lo=None, hi=None):
        r = self.rand(n) if n is not None else float(self.rand())
        if lo is None:
            return (r + 1.0) / 4294967296.0
        return lo + (hi - lo) * (r + 1.0) / 4294967296.0


class Distribution:
    """One of red's distribution objects: kind, seed and parameters."""

    def __init__(self, kind, seed, *params):
        self.kind, self.seed, self.params = kind, int(seed), tuple(float(p) for p in params)
        self.rr = RedRandom(seed)

    def draw(self, n):
        """The next n values (vectorised where red draws one uniform per value)."""
        k, p = self.kind, self.params
        if k == "uniform":
            return self.rr.uniform(n, p[0], p[1])
        if k == "exponential":
            u = self.rr.uniform(n)
            return np.array([-1.0 / p[0] * math.log(x) for x in u])
        if k == "rayleigh":
            u = self.rr.uniform(n)
            return np.array([p[0] * math.sqrt(-2.0 * math.log(x)) for x in u])
        if k == "normal":
            out = np.empty(n)
            for i in range(n):
                u = self.rr.uniform()
                r = self.rr.rand()
                out[i] = p[0] + p[1] * math.sqrt(-2.0 * math.log(u)) * math.cos(1.4629180792671596E-9 * (r + 1.0))
            return out
        if k == "power":
            x_min, x_max, power = p
            y_min = 0.0 if power == 0.0 else math.pow(x_min, power)
            y_max = 1.0 if power == 0.0 else math.pow(x_max, power)
            if y_min > y_max:
                y_min, y_max = y_max, y_min
            d_y, d_x = y_max - y_min, x_max - x_min
            area_max = d_x * d_y
            out = np.empty(n)
            for i in range(n):
                while True:
                    x = self.rr.uniform(None, 0.0, area_max) / d_y + x_min
                    y = self.rr.uniform(None, y_min, y_max)
                    if not y > math.pow(x, power):
                        break
                out[i] = x
            return out
        raise ValueError("unknown distribution " + k)


def parse_spec(text):
    """The harness's spec format: 'n type count', 'pp type item kind seed params...',
    'oe type element kind seed params...'.  Returns (counts, pp, oe) with pp[type][item]
    and oe[type][element] Distribution objects."""
    counts = [0] * BODY_TYPE_N
    pp = [dict() for _ in range(BODY_TYPE_N)]
    oe = [dict() for _ in range(BODY_TYPE_N)]
    for line in text.splitlines():
        f = line.split()
        if not f:
            continue
        t = int(f[1])
        if f[0] == "n":
            counts[t] = int(f[2])
        elif f[0] == "pp":
            pp[t][f[2]] = Distribution(f[3], f[4], *f[5:])
        elif f[0] == "oe":
            oe[t][f[2]] = Distribution(f[3], f[4], *f[5:])
    return counts, pp, oe


def calc_radius(m, density):
    """tools::calc_radius, tools.cpp:455-460."""
    return math.pow(1.0 / FOUR_PI_OVER_THREE * m / density, 1.0 / 3.0)


def calc_density(m, R):
    """tools::calc_density, tools.cpp:462-471."""
    return 0.0 if R == 0.0 else m / (FOUR_PI_OVER_THREE * (R * R * R))


def calc_mass(R, density):
    """tools::calc_mass, tools.cpp:473-478."""
    return FOUR_PI_OVER_THREE * (R * R * R) * density


def kepler_E(ecc, mean):
    """tools::kepler_equation_solver with red's tolerance 1e-8 (tools.cpp:715-755,
    called from calc_phase, :789-795), vectorised over bodies."""
    ecc = np.asarray(ecc, float)
    mean = np.asarray(mean, float).copy()
    trivial = (ecc == 0.0) | (mean == 0.0) | (mean == PI)
    s = mean > PI
    m2 = np.where(s, mean - PI, mean)
    E = m2 + ecc * (np.sin(m2)) / (1.0 - np.sin(m2 + ecc) + np.sin(m2))
    done = np.zeros(E.shape, bool)
    for _ in range(34):
        E1 = E - (E - ecc * np.sin(E) - m2) / (1.0 - ecc * np.cos(E))
        err = np.abs(E1 - E)
        E = np.where(done, E, E1)
        done |= err <= 1.0e-8
        if done.all():
            break
    # *E += (mean - *E) + PI: the reduced mean anomaly plus pi, not the solution
    E = np.where(s, E + ((m2 - E) + PI), E)
    return np.where(trivial, mean, E)


def calc_phase(mu, a, ecc, inc, peri, node, mean):
    """tools::calc_phase, tools.cpp:789-828, vectorised.  Returns r, v (n x 3)."""
    E = kepler_E(ecc, mean)
    v = 2.0 * np.arctan(np.sqrt((1.0 + ecc) / (1.0 - ecc)) * np.tan(E / 2.0))
    p = a * (1.0 - ecc * ecc)
    r = p / (1.0 + ecc * np.cos(v))
    kszi, eta = r * np.cos(v), r * np.sin(v)
    vkszi = -np.sqrt(mu / p) * np.sin(v)
    veta = np.sqrt(mu / p) * (ecc + np.cos(v))
    cw, sw, cO, sO, ci, si = np.cos(peri), np.sin(peri), np.cos(node), np.sin(node), np.cos(inc), np.sin(inc)
    P = np.stack([cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si], axis=1)
    Q = np.stack([-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si], axis=1)
    rv = np.stack([kszi * P[:, c] + eta * Q[:, c] for c in range(3)], axis=1)
    vv = np.stack([vkszi * P[:, c] + veta * Q[:, c] for c in range(3)], axis=1)
    return rv, vv


def transform_to_bc(mass, r, v, ids):
    """tools::transform_to_bc (tools.cpp:384-434): the barycentre summed from the
    last body to the first, inactive bodies skipped; r and v updated in place."""
    M0 = 0.0
    R0 = [0.0, 0.0, 0.0]
    V0 = [0.0, 0.0, 0.0]
    for j in range(len(mass) - 1, -1, -1):
        if ids[j] < 0:
            continue
        M0 += mass[j]
    for j in range(len(mass) - 1, -1, -1):
        if ids[j] < 0:
            continue
        for c in range(3):
            R0[c] += mass[j] * r[j, c]
            V0[c] += mass[j] * v[j, c]
    R0 = [x / M0 for x in R0]
    V0 = [x / M0 for x in V0]
    act = ids >= 0
    for c in range(3):
        r[act, c] -= R0[c]
        v[act, c] -= V0[c]


def populate(spec_text):
    """red's pipeline on one spec: populate_disk, the fix-up, calculate_phase,
    transform_to_bc, transform_time / transform_velocity.  Returns a dict of
    arrays (r, v: n x 3; mass, radius, density, cd, id, body_type; oe: n x 6)
    and dt (a thousandth of the shortest orbital period, k days)."""
    counts, pp, oe = parse_spec(spec_text)
    n = sum(counts)
    mass, radius, density, cd = (np.zeros(n) for _ in range(4))
    elems = np.zeros((n, 6))
    body_type = np.zeros(n, np.int32)
    i0 = 0
    for t in range(BODY_TYPE_N):
        c = counts[t]
        if c == 0:
            continue
        sl = slice(i0, i0 + c)
        body_type[sl] = t
        # every distribution is its own stream: a body's k-th quantity is the
        # k-th draw of that quantity's distribution
        drawn = {name: pp[t][name].draw(c) if name in pp[t] else np.zeros(c) for name in PP_NAMES}
        if t == TESTPARTICLE:
            drawn = {name: np.zeros(c) for name in PP_NAMES}
        elif t != SUPERPLANETESIMAL:
            has = {name: name in pp[t] for name in ("mass", "radius", "density")}
            for q in range(c):
                if not has["mass"] and has["radius"] and has["density"]:
                    drawn["mass"][q] = calc_mass(drawn["radius"][q], drawn["density"][q])
                elif not has["radius"] and has["mass"] and has["density"]:
                    drawn["radius"][q] = calc_radius(drawn["mass"][q], drawn["density"][q])
                elif not has["density"] and has["mass"] and has["radius"]:
                    drawn["density"][q] = calc_density(drawn["mass"][q], drawn["radius"][q])
                else:
                    raise ValueError("Missing physical parameters!")
        mass[sl], radius[sl], density[sl], cd[sl] = drawn["mass"], drawn["radius"], drawn["density"], drawn["cd"]
        first = 1 if t == STAR else 0          # the primary star keeps zero elements
        for k, name in enumerate(OE_NAMES):
            if name in oe[t] and c > first:
                elems[i0 + first:i0 + c, k] = oe[t][name].draw(c - first)
        i0 += c
    # the scenarios' fix-up after populate_disk (main.cu:2764-2781)
    i0 = 0
    for t in range(BODY_TYPE_N):
        for q in range(counts[t]):
            j = i0 + q
            if mass[j] > 0.0:
                if "density" not in pp[t] and "radius" in pp[t]:
                    density[j] = calc_density(mass[j], radius[j])
                if "radius" not in pp[t] and "density" in pp[t]:
                    radius[j] = calc_radius(mass[j], density[j])
        i0 += counts[t]
    ids = np.arange(1, n + 1, dtype=np.int32)
    r = np.zeros((n, 3))
    v = np.zeros((n, 3))
    mu = K2 * (mass[0] + mass[1:])
    r[1:], v[1:] = calc_phase(mu, elems[1:, 0], elems[1:, 1], elems[1:, 2], elems[1:, 3], elems[1:, 4], elems[1:, 5])
    a = elems[1:, 0]
    P = 6.283185307179586 * np.sqrt((a * a * a) / mu)     # tools::calc_orbital_period, tools.cpp:928-933
    dt = (P.min() / 1000.0 if n > 1 else 0.0) * K
    transform_to_bc(mass, r, v, ids)
    v /= K
    return {"r": r, "v": v, "mass": mass, "radius": radius, "density": density, "cd": cd, "id": ids,
            "body_type": body_type, "oe": elems}, dt
