"""Generates the golden fixtures in this directory from the reference's own code.

Runs oracle/_ref/ref_harness (built by oracle/ref_build.sh from the
unmodified suliaron/red.cuda sources) on small synthetic systems written in
red's input format, and stores inputs and the reference's outputs as .npz
files.  Only needed when the fixtures are regenerated; the tests read the
.npz files and never need the reference itself.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py initial    # only the disk generator's
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

rg = __graft_entry__.load_package()
HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
K = rg.ic.K


def run(args):
    subprocess.check_call([HARNESS] + args)


def rd(path):
    return open(path, "rb").read()


class Reader:
    def __init__(self, b):
        self.b, self.o = b, 0

    def take(self, dtype, n=1):
        dt = np.dtype(dtype)
        a = np.frombuffer(self.b, dt, n, self.o).copy()
        self.o += dt.itemsize * n
        return a

    def state(self):
        n = int(self.take("<u4")[0])
        playing = self.take("<u4", 7)
        inactive = self.take("<u4", 7)
        t = float(self.take("<f8")[0])
        r = self.take(rg.types.VAR4, n)
        v = self.take(rg.types.VAR4, n)
        p = self.take(rg.types.PARAM, n)
        md = self.take(rg.types.BMD, n)
        return dict(n=n, playing=playing, inactive=inactive, t=t, r=r, v=v, p=p, md=md)

    def events(self):
        n = int(self.take("<u4")[0])
        return self.take(rg.types.EVENT, n)


def si_system(n_pl=56, n_tp=4, seed=11):
    """Star + 4 protoplanets + n_pl bodies relabelled as protoplanets (all SI,
    which red's CPU path can integrate) + n_tp test particles."""
    rng = np.random.Generator(np.random.MT19937(seed))
    pl_a = rng.uniform(0.7, 1.5, n_pl)
    s = rg.ic.build_system(rng, pp_a=np.array([0.8, 1.0, 1.2, 1.4]), pp_mass=0.1 * rg.ic.EARTH_TO_SOLAR,
                           pl_a=pl_a, pl_mass=200.0 * rg.ic.EARTH_TO_SOLAR / n_pl, n_tp=n_tp)
    return s.relabel_all_SI()


def write(tmp, stem, s, t=0.0, dt=0.0, binary=False):
    info, data = rg.redio.write_system(tmp, stem, s, t=t, dt=dt, binary=binary)
    return info, data


def save(name, **kw):
    np.savez_compressed(os.path.join(HERE, name), **kw)
    print("wrote", name)


def case_accel(tmp):
    s = si_system()
    info, data = write(tmp, "acc", s)
    out = os.path.join(tmp, "acc.bin")
    run(["mode=accel", "dir=" + tmp, "info=" + info, "data=" + data, "out=" + out])
    R = Reader(rd(out))
    ok = R.take("<i4")[0]
    a = R.take(rg.types.VAR4, s.n)
    save("grav_cpu_si.npz", r=s.r, v=s.v, p=s.p, md=s.md, playing=s.playing, ok=ok, a=a)


def case_drag(tmp):
    s = rg.ic.config3(n_pp=3, n_pl=40, seed=5)
    keys = rg.ic.gas_disk_config3()
    keys["time_dependence"] = "exponential"
    keys["t0"] = 0.5
    keys["e_folding_time"] = 3.0
    rg.ic.write_gas_file(os.path.join(tmp, "gas.txt"), keys)
    info, data = write(tmp, "drag", s)
    out = os.path.join(tmp, "drag.bin")
    t = 1.25 * 365.25 * K
    run(["mode=accel", "dir=" + tmp, "info=" + info, "data=" + data, "out=" + out,
         "gasdir=" + tmp, "gas=gas.txt", "t=%r" % t])
    R = Reader(rd(out))
    R.take("<i4")
    R.take(rg.types.VAR4, s.n)
    d = R.take(rg.types.VAR4, s.n)
    gas = np.array([rg.ic.gas_params(keys)], dtype=rg.types.GAS)
    save("drag.npz", r=s.r, v=s.v, p=s.p, md=s.md, playing=s.playing, t=t, a=d, gas=gas,
         gas_text=np.frombuffer(open(os.path.join(tmp, "gas.txt"), "rb").read(), np.uint8))


def case_run(tmp, name, integrator, adaptive, tol, dt_days, nsteps, eftp=0):
    s = si_system()
    info, data = write(tmp, name, s, dt=dt_days * K)
    out = os.path.join(tmp, name + ".bin")
    run(["mode=run", "dir=" + tmp, "info=" + info, "data=" + data, "out=" + out,
         "integrator=%d" % integrator, "adaptive=%d" % adaptive, "tol=%r" % tol,
         "nsteps=%d" % nsteps, "eftp=%d" % eftp])
    R = Reader(rd(out))
    ns = int(R.take("<i4")[0])
    steps = R.take(np.dtype([("t", "<f8"), ("dt", "<f8"), ("dt_next", "<f8"), ("tried", "<u8"),
                             ("passed", "<u8"), ("failed", "<u8")]), ns)
    st = R.state()
    integ = R.take("<f8", 13)
    save(name + ".npz", r=s.r, v=s.v, p=s.p, md=s.md, playing=s.playing, dt0=dt_days * K,
         integrator=integrator, adaptive=adaptive, tol=tol, eftp=eftp, steps=steps,
         r_out=st["r"], v_out=st["v"], t_out=st["t"], integral=integ)


def collide_system(seed=7):
    """Small system with planted overlaps: a chain (3 bodies), a pair with a
    heavier second body, a test particle inside a protoplanet, and a body
    inside the star's enlarged radius."""
    s = si_system(n_pl=20, n_tp=3, seed=seed)
    r, p = s.r, s.p
    R = p["radius"]

    def place(j, i, frac):
        d = frac * (R[i] + R[j])
        r["x"][j], r["y"][j], r["z"][j] = r["x"][i] + d, r["y"][i], r["z"][i]

    place(10, 9, 0.6)
    place(11, 10, 0.5)       # chain 9-10-11
    p["mass"][13] = 3.0 * p["mass"][12]
    place(13, 12, 0.9)       # heavier second body survives
    place(s.n - 1, 2, 0.4)   # test particle inside protoplanet 2
    place(6, 0, 0.9)         # body inside the star
    return s


def case_collision(tmp):
    s = collide_system()
    info, data = write(tmp, "coll", s)
    out = os.path.join(tmp, "coll.bin")
    t = 12.5
    run(["mode=coll", "dir=" + tmp, "info=" + info, "data=" + data, "out=" + out,
         "factor=1.0", "t=%r" % t])
    R = Reader(rd(out))
    raw = R.events()
    sp = R.events()
    st = R.state()
    save("collision_cpu.npz", r=s.r, v=s.v, p=s.p, md=s.md, playing=s.playing, t=t, factor=1.0,
         raw=raw, sp=sp, r_out=st["r"], v_out=st["v"], p_out=st["p"], md_out=st["md"],
         inactive=st["inactive"])


def case_ejhc(tmp):
    s = si_system(n_pl=20, n_tp=3, seed=9)
    for c in "xyz":
        s.r[c][5] *= 30.0
        s.r[c][8] *= 0.05
        s.r[c][s.n - 2] *= 40.0
    info, data = write(tmp, "ejhc", s)
    out = os.path.join(tmp, "ejhc.bin")
    run(["mode=ejhc", "dir=" + tmp, "info=" + info, "data=" + data, "out=" + out,
         "ej=20.0", "hc=0.1", "t=3.0"])
    R = Reader(rd(out))
    raw = R.events()
    st = R.state()
    st2 = R.state()
    save("ejhc.npz", r=s.r, v=s.v, p=s.p, md=s.md, playing=s.playing, t=3.0, ej=20.0, hc=0.1, raw=raw,
         r_out=st["r"], v_out=st["v"], p_out=st["p"], md_out=st["md"], inactive=st["inactive"],
         rb_r=st2["r"], rb_md=st2["md"], rb_playing=st2["playing"], rb_n=st2["n"])


def case_integral(tmp):
    s = collide_system(seed=3)
    s.md["id"][4] *= -1      # an inactive body is left out of the sums
    info, data = write(tmp, "integ", s)
    out = os.path.join(tmp, "integ.bin")
    run(["mode=integral", "dir=" + tmp, "info=" + info, "data=" + data, "out=" + out])
    I = np.frombuffer(rd(out), "<f8").copy()
    save("integral.npz", r=s.r, v=s.v, p=s.p, md=s.md, playing=s.playing, integral=I)


def case_dump(tmp):
    s = si_system(n_pl=10, n_tp=2, seed=4)
    s.md["mig_type"][3] = 1
    s.md["mig_stop_at"][3] = 0.25
    info, data = write(tmp, "dump_in", s, t=1.5, dt=0.01)
    odir = os.path.join(tmp, "o")
    os.makedirs(odir, exist_ok=True)
    run(["mode=dump", "dir=" + tmp, "info=" + info, "data=" + data, "odir=" + odir])
    files = {}
    for f in ["ref_data.txt", "ref_data.info.txt", "ref_data.dat", "ref_data.info.dat"]:
        files[f.replace(".", "_")] = np.frombuffer(rd(os.path.join(odir, f)), np.uint8)
    save("formats.npz", r=s.r, v=s.v, p=s.p, md=s.md, playing=s.playing, t=1.5, dt=0.01,
         names=np.array(s.names), **files)


INITIAL_SPECS = {
    # star, 8 protoplanets (mass + density given: radius computed), 1000
    # planetesimals (log-uniform a: red's power law with power -1; drag
    # coefficient drawn), 20 test particles (exponential e, normal i)
    "initial_disk.npz": """n 0 1
pp 0 mass uniform 101 1.0 1.0
pp 0 radius uniform 102 0.004649 0.004649
pp 0 cd uniform 103 0.0 0.0
n 3 8
pp 3 mass uniform 111 1.0e-7 5.0e-7
pp 3 density uniform 112 336.0 336.0
oe 3 sma uniform 113 0.6 1.6
oe 3 ecc rayleigh 114 0.02
oe 3 inc rayleigh 115 0.01
oe 3 peri uniform 116 0.0 6.283185307179586
oe 3 node uniform 117 0.0 6.283185307179586
oe 3 mean uniform 118 0.0 6.283185307179586
n 5 1000
pp 5 mass uniform 121 1.0e-10 4.0e-9
pp 5 density uniform 122 200.0 500.0
pp 5 cd uniform 123 0.3 0.6
oe 5 sma power 124 0.5 3.0 -1.0
oe 5 ecc rayleigh 125 0.02
oe 5 inc rayleigh 126 0.01
oe 5 peri uniform 127 0.0 6.283185307179586
oe 5 node uniform 128 0.0 6.283185307179586
oe 5 mean uniform 129 0.0 6.283185307179586
n 6 20
oe 6 sma uniform 131 0.7 1.5
oe 6 ecc exponential 132 100.0
oe 6 inc normal 133 0.0 0.01
oe 6 peri uniform 134 0.0 6.283185307179586
oe 6 node uniform 135 0.0 6.283185307179586
oe 6 mean uniform 136 0.0 6.283185307179586
""",
    # the other fix-up branches: a giant planet with mass and radius given
    # (density computed), planetesimals with radius and density given (mass
    # computed), super-planetesimals (no fix-up) with all three given
    "initial_branches.npz": """n 0 1
pp 0 mass uniform 201 1.0 1.0
pp 0 radius uniform 202 0.004649 0.004649
n 1 2
pp 1 mass uniform 211 9.0e-4 1.0e-3
pp 1 radius uniform 212 4.0e-4 5.0e-4
oe 1 sma uniform 213 4.0 6.0
oe 1 ecc uniform 214 0.0 0.05
oe 1 inc uniform 215 0.0 0.02
oe 1 mean uniform 216 0.0 6.283185307179586
n 4 30
pp 4 mass uniform 221 1.0e-9 2.0e-9
pp 4 radius uniform 222 1.0e-6 2.0e-6
pp 4 density uniform 223 100.0 300.0
oe 4 sma uniform 224 1.0 2.0
oe 4 ecc rayleigh 225 0.05
n 5 300
pp 5 radius power 231 6.7e-9 6.7e-7 -1.0
pp 5 density uniform 232 336.0 336.0
pp 5 cd uniform 233 0.44 0.44
oe 5 sma uniform 234 0.5 4.0
oe 5 ecc rayleigh 235 0.01
oe 5 inc rayleigh 236 0.005
oe 5 peri uniform 237 0.0 6.283185307179586
oe 5 node uniform 238 0.0 6.283185307179586
oe 5 mean uniform 239 0.0 6.283185307179586
""",
}


def case_initial(tmp):
    """red.cuda.initial's own generator (oracle/_ref/initial_harness) on the specs above."""
    harness = os.path.join(ROOT, "oracle", "_ref", "initial_harness")
    for name, spec in INITIAL_SPECS.items():
        path = os.path.join(tmp, "spec.txt")
        open(path, "w").write(spec)
        out = os.path.join(tmp, "init.bin")
        subprocess.check_call([harness, path, out])
        R = Reader(rd(out))
        n = int(R.take("<u4")[0])
        dt = float(R.take("<f8")[0])
        r = R.take(rg.types.VAR4, n)
        v = R.take(rg.types.VAR4, n)
        p = R.take(rg.types.PARAM, n)
        md = R.take(rg.types.BMD, n)
        oe = R.take("<f8", 6 * n).reshape(n, 6)
        save(name, spec=np.frombuffer(spec.encode(), np.uint8), dt=dt, r=r, v=v, p=p, md=md, oe=oe)


CASES = ["accel", "drag", "runs", "collision", "ejhc", "integral", "dump", "initial"]


def main(cases=None):
    cases = cases or CASES
    if not os.path.exists(HARNESS) or not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "initial_harness")):
        subprocess.check_call([os.path.join(ROOT, "oracle", "ref_build.sh")])
    tmp = tempfile.mkdtemp(prefix="redgold")
    try:
        if "initial" in cases:
            case_initial(tmp)
        if "accel" not in cases:
            return
        case_accel(tmp)
        case_drag(tmp)
        case_run(tmp, "rk4_fixed", 4, 0, 0.0, 0.5, 40)
        case_run(tmp, "rk4_adaptive", 4, 1, 1e-10, 2.0, 25)
        case_run(tmp, "rkf78_adaptive", 8, 1, 1e-10, 5.0, 25)
        case_run(tmp, "rkf78_adaptive_tp", 8, 1, 1e-12, 5.0, 12, eftp=1)
        case_run(tmp, "rkf78_fixed", 8, 0, 0.0, 4.0, 20)
        case_run(tmp, "euler_fixed", 1, 0, 0.0, 0.05, 40)
        case_run(tmp, "rk2_fixed", 2, 0, 0.0, 0.2, 40)
        case_collision(tmp)
        case_ejhc(tmp)
        case_integral(tmp)
        case_dump(tmp)
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main(sys.argv[1:])
