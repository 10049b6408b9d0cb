"""CPU-side checks of the C ABI: the library builds, loads and exports every
entry point declared in include/redgb.h (no device calls)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "redgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(red_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_exports(rg):
    assert sorted(rg.EXPORTS) == declared_symbols()


def test_library_exports_every_declared_symbol(rg):
    rg.build()
    lib = rg.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.red_version().decode().startswith("redgb")


def test_struct_sizes_match_red(rg):
    import numpy as np
    from redgb.lib import Config, GasParams, SystemInfo
    assert ctypes.sizeof(GasParams) == rg.types.GAS.itemsize == 160
    assert rg.types.EVENT.itemsize == 432
    assert rg.types.BMD.itemsize == 24
    assert ctypes.sizeof(Config) > 0 and ctypes.sizeof(SystemInfo) > 0


def test_create_without_device_fails_loudly(rg):
    import torch
    if torch.cuda.is_available():
        import pytest
        pytest.skip("a device is present")
    s = rg.ic.config1(n_pl=8)
    try:
        rg.Sim(s, dt=0.1)
    except rg.RedError as e:
        assert e.code in (2, 8)
    else:
        raise AssertionError("red_create succeeded without a GPU")


def test_create_validates_inputs_before_touching_the_device(rg):
    """Argument checks run first, so they are testable without a GPU."""
    import numpy as np
    import torch
    if torch.cuda.is_available():
        import pytest
        pytest.skip("a device is present")
    s = rg.ic.config1(n_pl=8)
    bad = s.copy()
    bad.md["body_type"][1], bad.md["body_type"][6] = 5, 3      # not sorted by type
    for systems, code in [([s, s], 8), ([bad], 1)]:
        try:
            rg.Sim(systems, dt=0.1)
        except rg.RedError as e:
            assert e.code == code, (e, code)
        else:
            raise AssertionError("expected an error")
    for kw in (dict(integrator=3),      # no integrator of red has this code
               dict(gas_model=2)):      # red's FARGO disk throws in its constructor
        try:
            rg.Sim(s, dt=0.1, **kw)
        except rg.RedError as e:
            assert e.code == 6, (kw, e)
        else:
            raise AssertionError("expected RED_ERR_NOT_IMPLEMENTED for %r" % kw)
