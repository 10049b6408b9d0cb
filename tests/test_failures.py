"""Failure paths, injected on the host (no GPU fault, trap or hang).

CPU: truncated or corrupt body / info / parameter files give clean errors
from the Python readers (redio) and from the red-compatible driver
(redgb_run) before any device work.

GPU (the kernels bound every write, so none of these can fault):
* an event buffer of one record and a disk with many overlapping pairs:
  RED_ERR_EVENT_OVERFLOW, one record written, the state untouched, and the
  handle still integrates afterwards;
* a NaN position in one system of an ensemble: RED_ERR_NONFINITE for that
  system only; it stops, the other system keeps integrating with finite
  state.  (red has no such check: its controller would loop on the NaN error
  estimate, int_rungekutta8.cu:690-716.)
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "red.cuda_gb300", "_build", "redgb_run")


def vec(a):
    return np.stack([a["x"], a["y"], a["z"]], axis=1)


@pytest.mark.parametrize("binary", [False, True])
def test_redio_rejects_truncated_files(rg, tmp_path, binary):
    s = rg.ic.config1(seed=3, n_pl=40)
    info, data = rg.redio.write_system(str(tmp_path), "ic", s, binary=binary)
    raw = open(tmp_path / data, "rb").read()
    open(tmp_path / data, "wb").write(raw[:len(raw) // 2])
    with pytest.raises(ValueError, match="body records"):
        rg.redio.read_system(str(tmp_path), info, data)
    rawi = open(tmp_path / info, "rb").read()
    open(tmp_path / info, "wb").write(rawi[:20])
    with pytest.raises(ValueError, match="info record"):
        rg.redio.read_system(str(tmp_path), info, data)


def test_redio_rejects_corrupt_ascii_record(rg, tmp_path):
    s = rg.ic.config1(seed=3, n_pl=40)
    info, data = rg.redio.write_system(str(tmp_path), "ic", s)
    lines = open(tmp_path / data).read().splitlines()
    f = lines[7].split()
    f[10] = "1.0e-3x"
    lines[7] = " ".join(f)
    open(tmp_path / data, "w").write("\n".join(lines) + "\n")
    with pytest.raises(ValueError, match="malformed body record 7"):
        rg.redio.read_system(str(tmp_path), info, data)


@pytest.fixture(scope="module")
def driver(rg):
    rg.build()
    return DRIVER


def case(rg, d, binary):
    s = rg.ic.config1(seed=5, n_pl=64)
    info, data = rg.redio.write_system(str(d), "ic", s, t=0.0, dt=0.01, binary=binary)
    rg.redio.write_start_files(str(d), info, data)
    open(os.path.join(str(d), "param.txt"), "w").write("integrator = rkf8\ntolerance = 1e-10\nlength = 0.001\n")
    return info, data


def drive(d):
    return subprocess.run([DRIVER, "-idir", str(d), "-odir", str(d), "-p", "param.txt"], capture_output=True,
                          text=True, timeout=120)


@pytest.mark.parametrize("binary", [False, True])
def test_driver_rejects_truncated_body_file(driver, rg, tmp_path, binary):
    info, data = case(rg, tmp_path, binary)
    raw = open(tmp_path / data, "rb").read()
    open(tmp_path / data, "wb").write(raw[:len(raw) // 3])
    p = drive(tmp_path)
    assert p.returncode == 1
    assert ("Short binary data file" if binary else "Invalid body record") in p.stderr


def test_driver_rejects_corrupt_info_and_missing_files(driver, rg, tmp_path):
    info, data = case(rg, tmp_path, False)
    open(tmp_path / info, "w").write("0.0 0.01 zero 1 0 0 4 0 64 0\n")
    p = drive(tmp_path)
    assert p.returncode == 1 and "Invalid info record" in p.stderr
    os.remove(tmp_path / info)
    p = drive(tmp_path)
    assert p.returncode == 1 and "Cannot open" in p.stderr
    os.remove(tmp_path / "param.txt")
    p = drive(tmp_path)
    assert p.returncode == 1 and "Cannot open" in p.stderr


@pytest.mark.gpu
def test_event_buffer_overflow_is_reported(rg):
    s = rg.ic.config1(seed=31, n_pl=1500)
    with rg.Sim(s, dt=0.01, collision_factor=2000.0, event_capacity=1) as sim:
        before = sim.get_state(0)
        with pytest.raises(rg.lib.RedError) as e:
            sim.check_for_collision(cap=16)
        assert e.value.code == 3
        after = sim.get_state(0)
        assert np.array_equal(vec(after.r), vec(before.r)) and np.array_equal(vec(after.v), vec(before.v))
    with rg.Sim(s, dt=0.01 * rg.ic.K, collision_factor=0.0, event_capacity=1) as sim:
        for _ in range(3):
            sim.step()
        assert np.all(np.isfinite(vec(sim.get_state(0).r)))


@pytest.mark.gpu
def test_nonfinite_state_stops_only_its_system(rg):
    systems = [rg.ic.config1(seed=61, n_pl=300), rg.ic.config1(seed=62, n_pl=300)]
    with rg.Sim(systems, dt=1.0 * rg.ic.K, precision="mixed") as sim:
        bad = sim.get_state(1)
        bad.r["x"][7] = np.nan
        sim.set_state(1, bad)
        sim.launch_tries(5)
        with pytest.raises(rg.lib.RedError) as e:
            sim.synchronize()
        assert e.value.code == 5
        i0, i1 = sim.info(0), sim.info(1)
        assert i1.status == 5 and i0.status == 0
        assert i0.t > 0.0 and i0.n_passed >= 2
        assert np.all(np.isfinite(vec(sim.get_state(0).r)))
