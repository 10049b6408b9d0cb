"""red's file formats (ASCII / binary body and info records) against files
red itself wrote (tests/golden/formats.npz, from the reference harness's
dump mode, which calls red's file_util writers).

Writers: byte-identical to red's output.  In binary body records red writes
two ranges from uninitialised memory -- the bytes of the 30-byte name field
after its terminating NUL and the 4 padding bytes of body_metadata_t -- so
those are masked before the comparison.
Readers: the records read back equal the state red dumped, field by field.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "formats.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def golden_system(rg, g):
    s = rg.types.System(g["r"].copy(), g["v"].copy(), g["p"].copy(), g["md"].copy(), g["playing"].copy(),
                        [str(x) for x in g["names"]])
    return s


def test_ascii_writers_byte_identical(rg, gold, tmp_path):
    s = golden_system(rg, gold)
    info, data = rg.redio.write_system(str(tmp_path), "out", s, t=float(gold["t"]), dt=float(gold["dt"]))
    assert open(tmp_path / data, "rb").read() == bytes(gold["ref_data_txt"])
    assert open(tmp_path / info, "rb").read() == bytes(gold["ref_data_info_txt"])


def test_binary_writers_byte_identical(rg, gold, tmp_path):
    s = golden_system(rg, gold)
    info, data = rg.redio.write_system(str(tmp_path), "out", s, t=float(gold["t"]), dt=float(gold["dt"]),
                                       binary=True)
    mine = np.frombuffer(open(tmp_path / data, "rb").read(), np.uint8).reshape(-1, 134).copy()
    ref = bytes(gold["ref_data_dat"])
    ref = np.frombuffer(ref, np.uint8).reshape(-1, 134).copy()
    for a in (mine, ref):
        a[:, 42:46] = 0                           # body_metadata_t padding
        for row in a:
            row[int(np.argmax(row[:30] == 0)):30] = 0   # name bytes after the NUL
    assert np.array_equal(mine, ref)
    assert open(tmp_path / info, "rb").read() == bytes(gold["ref_data_info_dat"])


@pytest.mark.parametrize("ext", ["txt", "dat"])
def test_readers_round_trip_red_files(rg, gold, tmp_path, ext):
    stem = "ref_data"
    open(tmp_path / ("%s.%s" % (stem, ext)), "wb").write(bytes(gold["ref_data_" + ext]))
    open(tmp_path / ("%s.info.%s" % (stem, ext)), "wb").write(bytes(gold["ref_data_info_" + ext]))
    s, t, dt, dt_cpu = rg.redio.read_system(str(tmp_path), "%s.info.%s" % (stem, ext), "%s.%s" % (stem, ext))
    assert t == float(gold["t"]) and dt == float(gold["dt"])
    assert list(s.playing) == list(gold["playing"])
    for f in ("x", "y", "z"):
        assert np.array_equal(s.r[f], gold["r"][f])
        assert np.array_equal(s.v[f], gold["v"][f])
    for f in gold["p"].dtype.names:
        assert np.array_equal(s.p[f], gold["p"][f])
    for f in ("id", "body_type", "mig_type", "mig_stop_at"):
        assert np.array_equal(s.md[f], gold["md"][f])
    assert s.names == [str(x) for x in gold["names"]]
