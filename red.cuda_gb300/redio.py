"""red's input / snapshot file formats, host side (numpy).

ASCII body record (15 fields, file_util.cpp:355-381 writer, 593-633 reader):
    name id type mig_type mig_stop_at mass radius density cd x y z vx vy vz
ASCII info record (file_util.cpp:325-341 writer, 562-571 reader):
    t dt dt_CPU n_s n_gp n_rp n_pp n_spl n_pl n_tp
Binary body record: 30-byte name, 24-byte body_metadata_t, 32-byte param_t,
3 doubles r, 3 doubles v = 134 bytes (file_util.cpp:383-390).
Binary info record: t, dt (doubles), dt_CPU (uint32), 7 x uint32 = 48 bytes
(file_util.cpp:343-353).
``start_files.txt`` holds the info file name on line 1 and the data file name
on line 2 (options.cpp:228-246).

The writers use the same field widths as red (setw 30/8/2/25, precision 16,
scientific) so that a file written here is byte-identical to one red writes.
Time is stored in red's code unit (1/k day) and velocities in AU per code
unit.
"""
import os
import struct

import numpy as np

from .types import BMD, PARAM, VAR4, System


def _fmt_d(x):
    return "%25.16e" % x


def write_info_ascii(path, t, dt, dt_cpu, counts):
    s = "%s %s %10d " % (_fmt_d(t), _fmt_d(dt), dt_cpu)
    s += "".join("%8d " % c for c in counts)
    with open(path, "w") as f:
        f.write(s)


def write_data_ascii(path, sysm):
    lines = []
    for i in range(sysm.n):
        if sysm.md["id"][i] < 0:
            continue
        name = sysm.names[i] if sysm.names is not None else "body%d" % i
        lines.append("%30s %8d %2d %2d %s %s %s %s %s %s %s %s %s %s %s\n" % (
            name, sysm.md["id"][i], sysm.md["body_type"][i], sysm.md["mig_type"][i],
            _fmt_d(sysm.md["mig_stop_at"][i]), _fmt_d(sysm.p["mass"][i]), _fmt_d(sysm.p["radius"][i]),
            _fmt_d(sysm.p["density"][i]), _fmt_d(sysm.p["cd"][i]),
            _fmt_d(sysm.r["x"][i]), _fmt_d(sysm.r["y"][i]), _fmt_d(sysm.r["z"][i]),
            _fmt_d(sysm.v["x"][i]), _fmt_d(sysm.v["y"][i]), _fmt_d(sysm.v["z"][i])))
    with open(path, "w") as f:
        f.writelines(lines)


def write_info_binary(path, t, dt, dt_cpu, counts):
    with open(path, "wb") as f:
        f.write(struct.pack("<ddI7I", t, dt, dt_cpu, *[int(c) for c in counts]))


def write_data_binary(path, sysm):
    with open(path, "wb") as f:
        for i in range(sysm.n):
            if sysm.md["id"][i] < 0:
                continue
            name = (sysm.names[i] if sysm.names is not None else "body%d" % i).encode()[:30]
            f.write(name.ljust(30, b"\0"))
            f.write(sysm.md[i:i + 1].tobytes())
            f.write(sysm.p[i:i + 1].tobytes())
            f.write(struct.pack("<3d", sysm.r["x"][i], sysm.r["y"][i], sysm.r["z"][i]))
            f.write(struct.pack("<3d", sysm.v["x"][i], sysm.v["y"][i], sysm.v["z"][i]))


def write_system(dirname, stem, sysm, t=0.0, dt=0.0, dt_cpu=0, binary=False):
    """Writes <stem>.info.<ext> and <stem>.<ext>; returns (info_name, data_name)."""
    ext = "dat" if binary else "txt"
    info = "%s.info.%s" % (stem, ext)
    data = "%s.%s" % (stem, ext)
    counts = sysm.active_counts()
    if binary:
        write_info_binary(os.path.join(dirname, info), t, dt, dt_cpu, counts)
        write_data_binary(os.path.join(dirname, data), sysm)
    else:
        write_info_ascii(os.path.join(dirname, info), t, dt, dt_cpu, counts)
        write_data_ascii(os.path.join(dirname, data), sysm)
    return info, data


def read_info(path):
    """(t, dt, dt_CPU, counts[7]) of an info record; ValueError on a short or
    malformed record (red's reader would read garbage, file_util.cpp:325-353)."""
    if path.endswith(".dat"):
        with open(path, "rb") as f:
            raw = f.read(48)
        if len(raw) < 48:
            raise ValueError("%s: binary info record of %d bytes, expected 48" % (path, len(raw)))
        t, dt, dt_cpu, *counts = struct.unpack("<ddI7I", raw)
        return t, dt, dt_cpu, np.array(counts, np.uint32)
    tok = open(path).read().split()
    if len(tok) < 10:
        raise ValueError("%s: info record of %d fields, expected 10" % (path, len(tok)))
    try:
        return float(tok[0]), float(tok[1]), int(tok[2]), np.array([int(x) for x in tok[3:10]], np.uint32)
    except ValueError as e:
        raise ValueError("%s: malformed info record (%s)" % (path, e)) from None


def read_data(path, n):
    r = np.zeros(n, VAR4)
    v = np.zeros(n, VAR4)
    p = np.zeros(n, PARAM)
    md = np.zeros(n, BMD)
    names = []
    if path.endswith(".dat"):
        raw = open(path, "rb").read()
        rec = 134
        if len(raw) < rec * n:
            raise ValueError("%s: %d bytes hold %d of the %d body records" % (path, len(raw), len(raw) // rec, n))
        for i in range(n):
            b = raw[i * rec:(i + 1) * rec]
            names.append(b[:30].split(b"\0")[0].decode())
            md[i] = np.frombuffer(b[30:54], BMD)[0]
            p[i] = np.frombuffer(b[54:86], PARAM)[0]
            x = struct.unpack("<6d", b[86:134])
            r[i] = (x[0], x[1], x[2], 0.0)
            v[i] = (x[3], x[4], x[5], 0.0)
    else:
        tok = open(path).read().split()
        if len(tok) < 15 * n:
            raise ValueError("%s: %d fields hold %d of the %d body records" % (path, len(tok), len(tok) // 15, n))
        for i in range(n):
            f = tok[i * 15:(i + 1) * 15]
            names.append(f[0][:30])
            try:
                md[i] = (int(f[1]), int(f[2]), int(f[3]), float(f[4]))
                p[i] = tuple(float(x) for x in f[5:9])
                r[i] = (float(f[9]), float(f[10]), float(f[11]), 0.0)
                v[i] = (float(f[12]), float(f[13]), float(f[14]), 0.0)
            except ValueError as e:
                raise ValueError("%s: malformed body record %d (%s)" % (path, i, e)) from None
    return r, v, p, md, names


def read_system(dirname, info, data):
    t, dt, dt_cpu, counts = read_info(os.path.join(dirname, info))
    n = int(counts.sum())
    r, v, p, md, names = read_data(os.path.join(dirname, data), n)
    return System(r, v, p, md, counts, names), t, dt, dt_cpu


def write_start_files(dirname, info, data):
    with open(os.path.join(dirname, "start_files.txt"), "w") as f:
        f.write(info + "\n" + data + "\n")
