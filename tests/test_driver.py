"""redgb_run, the command-line driver with red's interface (options,
parameter file, start files, body / info / integral records), over the C ABI.

CPU tests check the refusals that come before any device work.  The GPU test
runs a small disk through the driver and through the library directly with
the same settings in FP64_EXACT: the final snapshot the driver writes in red's
ASCII format (17 significant digits) equals the library's state bit for bit,
the snapshot numbering and start_files.txt follow red's conventions, and a
restart from the driver's own output continues the numbering.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "red.cuda_gb300", "_build", "redgb_run")


@pytest.fixture(scope="module")
def driver(rg):
    rg.build()
    return DRIVER


def write_case(rg, d, params):
    s = rg.ic.config1(seed=5, n_pl=64)
    info, data = rg.redio.write_system(str(d), "ic", s, t=0.0, dt=0.01)
    rg.redio.write_start_files(str(d), info, data)
    with open(os.path.join(str(d), "param.txt"), "w") as f:
        for k, v in params.items():
            f.write("%s = %s\n" % (k, v))
    return s


def run(driver, *args):
    return subprocess.run([driver, *args], capture_output=True, text=True, timeout=600)


def test_usage(driver):
    p = run(driver, "-h")
    assert p.returncode == 0 and "usage: redgb_run" in p.stdout


def test_parameter_file_required(driver):
    p = run(driver)
    assert p.returncode == 1 and "parameter file" in p.stderr


def write_param_text(d, text):
    with open(os.path.join(str(d), "param.txt"), "w") as f:
        f.write(text)


def test_malformed_line_rejected(driver, rg, tmp_path):
    """parameter::parse throws on a line without a key = value pair (parameter.cpp:96)."""
    write_case(rg, tmp_path, {})
    write_param_text(tmp_path, "integrator = rkf8\ntolerance 1e-10\n")
    p = run(driver, "-idir", str(tmp_path), "-odir", str(tmp_path), "-p", "param.txt")
    assert p.returncode == 1 and "Invalid key/value pair: tolerance 1e-10." in p.stderr


def test_invalid_number_rejected(driver, rg, tmp_path):
    write_case(rg, tmp_path, {})
    write_param_text(tmp_path, "tolerance = 1e-1O\n")
    p = run(driver, "-idir", str(tmp_path), "-odir", str(tmp_path), "-p", "param.txt")
    assert p.returncode == 1 and "Invalid number at: tolerance" in p.stderr


@pytest.mark.parametrize("integrator", ["E", "Euler", "RK2", "Runge-Kutta4", "RKF8"])
def test_keys_and_values_case_insensitive(driver, rg, tmp_path, integrator):
    """Keys and the integrator / representation values are lower-cased as red
    does (parameter.cpp:108, 120, 136); every integrator of red is taken.  The
    parse comes before any device work: without a GPU the run stops later, at
    the device, never at the parameter file."""
    write_case(rg, tmp_path, {})
    write_param_text(tmp_path, "Integrator = %s\nTOLERANCE = 1e-10\nLength = 0.001\nODR = Text\n" % integrator)
    p = run(driver, "-idir", str(tmp_path), "-odir", str(tmp_path), "-p", "param.txt")
    assert "Invalid" not in p.stderr, p.stderr
    assert p.returncode == 0 or "device" in p.stderr.lower() or "cuda" in p.stderr.lower(), p.stderr


def test_invalid_parameter_refused(driver, rg, tmp_path):
    write_case(rg, tmp_path, {"no such key": "1"})
    p = run(driver, "-idir", str(tmp_path), "-odir", str(tmp_path), "-p", "param.txt")
    assert p.returncode == 1 and "Invalid parameter" in p.stderr


@pytest.mark.gpu
def test_driver_run_matches_library_and_restarts(driver, rg, tmp_path):
    params = {"integrator": "rkf8", "tolerance": "1e-10", "length": "0.02", "output interval": "0.005",
              "odr": "text"}
    s = write_case(rg, tmp_path, params)
    out = tmp_path / "out"
    out.mkdir()
    p = run(driver, "-idir", str(tmp_path), "-odir", str(out), "-p", "param.txt", "-prec", "fp64_exact")
    assert p.returncode == 0, p.stderr
    snaps = sorted(f for f in os.listdir(out) if f.startswith("data_") and not f.endswith(".info.txt"))
    assert snaps[0] == "data_000000000.txt" and len(snaps) >= 4
    start = open(out / "start_files.txt").read().split()
    assert start == [snaps[-1].replace(".txt", ".info.txt"), snaps[-1]]
    assert len(open(out / "integral.txt").read().splitlines()) == len(snaps)
    final, t_final, _, _ = rg.redio.read_system(str(out), start[0], start[1])

    K = rg.ic.K
    with rg.Sim(s, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=0.01, precision="fp64_exact",
                output_interval=0.005 * 365.25 * K, length=0.02 * 365.25 * K) as sim:
        while sim.info(0).active:
            sim.step()
        ref = sim.get_state(0)
        t_ref = sim.info(0).t
    assert t_final == t_ref
    for f in "xyz":
        assert np.array_equal(final.r[f], ref.r[f])
        assert np.array_equal(final.v[f], ref.v[f])

    # restart from the driver's own output: the numbering continues
    with open(out / "param.txt", "w") as f:
        for k, v in dict(params, length="0.006").items():
            f.write("%s = %s\n" % (k, v))
    p = run(driver, "-idir", str(out), "-odir", str(out), "-p", "param.txt", "-prec", "fp64_exact")
    assert p.returncode == 0, p.stderr
    snaps2 = sorted(f for f in os.listdir(out) if f.startswith("data_") and not f.endswith(".info.txt"))
    assert len(snaps2) > len(snaps)
    n_last = int(snaps[-1][5:14])
    assert int(snaps2[len(snaps)][5:14]) == n_last + 1


@pytest.mark.gpu
def test_driver_euler_from_parameter_file(driver, rg, tmp_path):
    """Euler chosen in the parameter file (upper case) runs at the fixed initial
    step and ends where the library's red-exact Euler run ends, bit for bit."""
    s = write_case(rg, tmp_path, {})
    write_param_text(tmp_path, "INTEGRATOR = E\nlength = 0.002\nodr = text\n")
    out = tmp_path / "out"
    out.mkdir()
    p = run(driver, "-idir", str(tmp_path), "-odir", str(out), "-p", "param.txt", "-prec", "fp64_exact")
    assert p.returncode == 0, p.stderr
    start = open(out / "start_files.txt").read().split()
    final, t_final, _, _ = rg.redio.read_system(str(out), start[0], start[1])
    K = rg.ic.K
    with rg.Sim(s, integrator="euler", adaptive=False, dt=0.01, precision="fp64_exact",
                length=0.002 * 365.25 * K) as sim:
        while sim.info(0).active:
            sim.step()
        ref = sim.get_state(0)
        t_ref = sim.info(0).t
    assert t_final == t_ref
    for f in "xyz":
        assert np.array_equal(final.r[f], ref.r[f]) and np.array_equal(final.v[f], ref.v[f])
