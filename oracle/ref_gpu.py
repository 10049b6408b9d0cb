"""red's own GPU path, run as a checker and as a baseline -- TEST INFRASTRUCTURE.

red.cuda's production path is FP64 CUDA: ``calc_grav_accel_naive`` launched
once per body class (``src/red.cuda/pp_disk.cu:373-416, 1014-1045``), the
``rk8_kernel`` / ``rk4_kernel`` stage sums (``int_rungekutta8.cu:80-274``),
thrust's ``max_element`` for the error norm and the host step controller
(``int_rungekutta8.cu:635-716``), with a device synchronisation after every
launch (``red_macro.h:33, 62-90``).  This module drives that code, unmodified,
through ``oracle/ref_harness.cu`` with ``dev=gpu``:

* the parity tests pin the oracle's GPU semantics (NSI / NI bounds, the star
  taken as i in the collision loop) and this library's FP64_EXACT mode
  against red's own kernels on the same inputs;
* ``bench.py`` times it as the "plain FP64 single-system GPU path".

The harness must be built where the GPU is: ``oracle/ref_stage.sh`` stages
an unmodified copy of red's sources under the git-ignored ``baseline/_ref/``,
and ``build()`` compiles it there with ``oracle/ref_build.sh`` into
``oracle/_ref/box/``.  Only ``tests/`` and ``bench.py``'s baseline legs use
this module; the library never does.
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STAGED = os.path.join(ROOT, "baseline", "_ref", "red.cuda")
OUT = os.path.join(HERE, "_ref", "box")
HARNESS = os.path.join(OUT, "ref_harness")


def available():
    """True when the staged copy of red's sources is present."""
    return os.path.isdir(os.path.join(STAGED, "src", "red.cuda"))


def _is_native(path):
    """The binary exists and was built for this machine's CPU architecture."""
    if not os.path.exists(path):
        return False
    import platform
    with open(path, "rb") as f:
        head = f.read(20)
    if head[:4] != b"\x7fELF":
        return False
    machine = int.from_bytes(head[18:20], "little")
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return want is None or machine == want


def build():
    """Builds oracle/_ref/box/ref_harness from the staged sources (about 20 s)."""
    if not available():
        raise RuntimeError("red's sources are not staged under baseline/_ref (oracle/ref_stage.sh)")
    if _is_native(HARNESS):
        newest = max(os.path.getmtime(os.path.join(d, f)) for d, _, fs in os.walk(STAGED) for f in fs)
        newest = max(newest, os.path.getmtime(os.path.join(HERE, "ref_harness.cu")))
        if os.path.getmtime(HARNESS) >= newest:
            return HARNESS
    if os.path.isdir(os.path.join(OUT, "obj")):
        # objects of another architecture (the copy came from another machine)
        for f in os.listdir(os.path.join(OUT, "obj")):
            os.remove(os.path.join(OUT, "obj", f))
    env = dict(os.environ, RED_REFERENCE=STAGED, RED_REF_OUT=OUT)
    subprocess.check_call([os.path.join(HERE, "ref_build.sh")], env=env, stdout=subprocess.DEVNULL)
    return HARNESS


class Reader:
    """Parses the harness's raw little-endian records."""

    def __init__(self, b, types):
        self.b, self.o, self.T = b, 0, types

    def take(self, dtype, n=1):
        dt = np.dtype(dtype)
        a = np.frombuffer(self.b, dt, n, self.o).copy()
        self.o += dt.itemsize * n
        return a

    def state(self):
        T = self.T
        n = int(self.take("<u4")[0])
        playing = self.take("<u4", 7)
        inactive = self.take("<u4", 7)
        t = float(self.take("<f8")[0])
        r = self.take(T.VAR4, n)
        v = self.take(T.VAR4, n)
        p = self.take(T.PARAM, n)
        md = self.take(T.BMD, n)
        return dict(n=n, playing=playing, inactive=inactive, t=t, r=r, v=v, p=p, md=md)

    def events(self):
        n = int(self.take("<u4")[0])
        return self.take(self.T.EVENT, n)


STEP = np.dtype([("t", "<f8"), ("dt", "<f8"), ("dt_next", "<f8"), ("tried", "<u8"), ("passed", "<u8"),
                 ("failed", "<u8")])


def _write(rg, tmp, s, dt):
    """s in red's binary format with every playing body, inactive ones (id < 0)
    included: red keeps them in its arrays and skips them in its loops."""
    info, data = "in.info.dat", "in.dat"
    rg.redio.write_info_binary(os.path.join(tmp, info), 0.0, dt, 0, s.playing)
    with open(os.path.join(tmp, data), "wb") as f:
        for i in range(s.n):
            f.write(("body%d" % i).encode().ljust(30, b"\0"))
            f.write(s.md[i:i + 1].tobytes())
            f.write(s.p[i:i + 1].tobytes())
            f.write(np.array([s.r["x"][i], s.r["y"][i], s.r["z"][i], s.v["x"][i], s.v["y"][i], s.v["z"][i]],
                             "<f8").tobytes())
    return info, data


def _run(rg, s, args, dt=0.0, gas_keys=None, timeout=3600):
    """Writes s in red's binary format, runs the harness on it, returns the output bytes."""
    with tempfile.TemporaryDirectory(prefix="redgpu") as tmp:
        info, data = _write(rg, tmp, s, dt)
        out = os.path.join(tmp, "out.bin")
        tout = os.path.join(tmp, "time.txt")
        cmd = [HARNESS, "dev=gpu", "dir=" + tmp, "info=" + info, "data=" + data, "out=" + out,
               "tout=" + tout] + list(args)
        if gas_keys is not None:
            rg.ic.write_gas_file(os.path.join(tmp, "gas.txt"), gas_keys)
            cmd += ["gasdir=" + tmp, "gas=gas.txt"]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, timeout=timeout)
        timing = open(tout).read().split() if os.path.exists(tout) else None
        return open(out, "rb").read(), timing


def accel(rg, s, t=0.0, gas_keys=None, tpb=None):
    """red's calc_dydx(1, ...) on the GPU: gravity of every class plus drag (n var4)."""
    args = ["mode=accel", "t=%r" % t] + (["tpb=%d" % tpb] if tpb else [])
    b, _ = _run(rg, s, args, gas_keys=gas_keys)
    R = Reader(b, rg.types)
    assert int(R.take("<i4")[0]) == 1
    return R.take(rg.types.VAR4, s.n)


def run(rg, s, integrator, dt, nsteps, adaptive=False, tol=1e-10, eftp=False, gas_keys=None, tpb=None):
    """nsteps of red's integrator on the GPU.  Returns the per-step record
    (t, dt, dt_next, tried, passed, failed), the final state, red's integrals,
    the step loop's wall seconds and the threads per block used."""
    kind = {"euler": 1, "rk2": 2, "rk4": 4, "rkf78": 8}[integrator]
    args = ["mode=run", "integrator=%d" % kind, "adaptive=%d" % int(adaptive), "tol=%r" % tol,
            "nsteps=%d" % nsteps, "eftp=%d" % int(eftp)] + (["tpb=%d" % tpb] if tpb else [])
    b, timing = _run(rg, s, args, dt=dt, gas_keys=gas_keys)
    R = Reader(b, rg.types)
    ns = int(R.take("<i4")[0])
    steps = R.take(STEP, ns)
    st = R.state()
    integ = R.take("<f8", 13)
    return dict(steps=steps, state=st, integral=integ, seconds=float(timing[0]), tpb=int(timing[1]))


def collisions(rg, s, factor, t=0.0):
    """red's GPU collision check on s.  The caller must have counted the pairs
    (at most s.n fit red's unchecked event buffer)."""
    b, _ = _run(rg, s, ["mode=coll", "factor=%r" % factor, "t=%r" % t])
    return Reader(b, rg.types).events()
