"""The C++ host driver (funwave-tvd_gb300/host/fw_main.cpp), which has the
shape of the reference's main program over the C ABI.

CPU: input.txt parsing and the DEPTH_TYPE DATA / FLAT / SLOPE depths
(init.F:684-760), written as dep.out in PutFile's ASCII format (io.F:4895-
4921: Mglob values per line, E16.6E4), in --dry-run mode (no GPU).
GPU: a short run writes eta_00001 (the initial state) and one file per
PLOT_INTV, and its last file equals the Python Solver's state at the same
time to the printed precision.
"""
import os
import subprocess

import numpy as np
import pytest


def e16_6e4(v):
    """Fortran E16.6E4 of float(v)."""
    v = float(np.float32(v))
    if v == 0.0:
        return "%16s" % "0.000000E+0000"
    m, e = ("%.5E" % v).split("E")
    neg = m.startswith("-")
    digits = m.lstrip("-").replace(".", "")
    return "%16s" % ("%s0.%sE%s%04d" % ("-" if neg else "", digits, "-" if int(e) + 1 < 0 else "+",
                                        abs(int(e) + 1)))


def read_put_file(path):
    rows = []
    for line in open(path):
        line = line.rstrip("\n")
        rows.append([float(line[k:k + 16]) for k in range(0, len(line), 16)])
    return np.array(rows).T  # (Mglob, Nglob)


def _write_input(d, extra):
    keys = {"Mglob": 24, "Nglob": 16, "DX": 2.0, "DY": 2.0, "RESULT_FOLDER": d + "/"}
    keys.update(extra)
    with open(os.path.join(d, "input.txt"), "w") as f:
        f.write("! test deck\n")
        for k, v in keys.items():
            f.write("%s = %s   ! comment\n" % (k, v))
        f.write("Mglob = 999\n")  # a later duplicate is ignored
    return keys


def _driver(fw):
    fw.build()
    return fw.solver.driver_path()


def _dry(fw, d):
    r = subprocess.run([_driver(fw), os.path.join(d, "input.txt"), "--dry-run"], capture_output=True, text=True,
                       cwd=d)
    assert r.returncode == 0, r.stderr
    return read_put_file(os.path.join(d, "dep.out"))


def test_format_matches_fortran_e16_6e4():
    assert e16_6e4(0.0) == "  0.000000E+0000"
    assert e16_6e4(1.0) == "  0.100000E+0001"
    assert e16_6e4(-0.00123456789) == " -0.123457E-0002"
    assert e16_6e4(999999.0) == "  0.999999E+0006"


def test_depth_data_file(fw, tmp_path):
    d = str(tmp_path)
    rng = np.random.default_rng(5)
    depth = rng.uniform(-1.0, 8.0, size=(24, 16))
    with open(os.path.join(d, "depth.txt"), "w") as f:
        for j in range(16):
            f.write(" ".join("%.6f" % depth[i, j] for i in range(24)) + "\n")
    _write_input(d, {"DEPTH_TYPE": "DATA", "DEPTH_FILE": os.path.join(d, "depth.txt")})
    out = _dry(fw, d)
    assert out.shape == (24, 16)
    written = np.array([[float("%.6f" % depth[i, j]) for j in range(16)] for i in range(24)])
    # E16.6 keeps six significant digits of the float value
    assert np.allclose(out, written, rtol=6e-6, atol=0.0)
    line = open(os.path.join(d, "dep.out")).readline().rstrip("\n")
    assert len(line) == 16 * 24
    assert line[:16] == e16_6e4(float("%.6f" % depth[0, 0]))


def test_depth_flat_and_slope(fw, tmp_path):
    d = str(tmp_path)
    _write_input(d, {"DEPTH_TYPE": "FLAT", "DEPTH_FLAT": 7.5})
    assert np.all(_dry(fw, d) == 7.5)
    _write_input(d, {"DEPTH_TYPE": "SLOPE", "DEPTH_FLAT": 6.0, "SLP": 0.05, "Xslp": 11.0})
    out = _dry(fw, d)
    i0 = int(11.0 / 2.0) + 1  # Fortran INT(Xslp/DX)+1, 1-based
    I = np.arange(1, 25)
    expect = np.where(I >= i0, 6.0 - 0.05 * (I - i0) * 2.0, 6.0)
    assert np.allclose(out, expect[:, None], rtol=6e-6)


@pytest.mark.gpu
def test_driver_run_matches_solver(fw, tmp_path):
    d = str(tmp_path)
    extra = {"DEPTH_TYPE": "SLOPE", "DEPTH_FLAT": 3.0, "SLP": 0.04, "Xslp": 20.0, "WAVEMAKER": "WK_REG",
             "AMP_WK": 0.05, "Tperiod": 3.0, "DEP_WK": 3.0, "Xc_WK": 10.0, "Time_ramp": 1.0,
             "TOTAL_TIME": 3.0, "PLOT_INTV": 1.0, "PERIODIC": "T", "MinDepth": 0.01}
    keys = _write_input(d, extra)
    r = subprocess.run([_driver(fw), os.path.join(d, "input.txt")], capture_output=True, text=True, cwd=d,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    files = sorted(f for f in os.listdir(d) if f.startswith("eta_"))
    assert files[0] == "eta_00001" and len(files) >= 3
    assert np.all(read_put_file(os.path.join(d, "eta_00001")) == 0.0)
    times = np.loadtxt(os.path.join(d, "time_dt.out"), ndmin=2)
    assert times.shape[0] == len(files)
    # the same run through the Python Solver, to the last file's time
    p = {k: v for k, v in keys.items() if k not in ("RESULT_FOLDER",)}
    p["PERIODIC"] = True
    i0 = int(20.0 / 2.0) + 1
    I = np.arange(1, 25)
    depth = np.repeat(np.where(I >= i0, 3.0 - 0.04 * (I - i0) * 2.0, 3.0)[:, None], 16, axis=1)
    s = fw.Solver(fw.with_defaults(p), precision="FP64")
    s.init(np.asfortranarray(depth))
    while s.scalar("TIME") < times[-1, 0] * (1.0 - 1e-8):  # the printed TIME has 10 digits
        s.step(1)
    assert abs(s.scalar("TIME") - times[-1, 0]) <= 1e-6 * times[-1, 0]
    last = read_put_file(os.path.join(d, files[-1]))
    eta = s.get("Eta")[3:-3, 3:-3]
    assert np.abs(eta).max() > 1e-4
    assert np.allclose(last, eta.astype(np.float32), rtol=6e-6, atol=1e-12)
    s.close()


@pytest.mark.gpu
def test_driver_binary_fields_and_stations(fw, tmp_path):
    """FIELD_IO_TYPE = BINARY writes the interior in Fortran order as double
    (FP64), equal to the solver's state; STATIONS samples eta, u, v at the
    station cells each PLOT_INTV_STATION (zeros on dry cells)."""
    d = str(tmp_path)
    with open(os.path.join(d, "stations.txt"), "w") as f:
        f.write("6 5\n24 8\n30 9\n")  # the last one lies outside the 24 x 16 grid
    extra = {"DEPTH_TYPE": "SLOPE", "DEPTH_FLAT": 3.0, "SLP": 0.2, "Xslp": 20.0, "WAVEMAKER": "WK_REG",
             "AMP_WK": 0.05, "Tperiod": 3.0, "DEP_WK": 3.0, "Xc_WK": 10.0, "Time_ramp": 1.0,
             "TOTAL_TIME": 3.0, "PLOT_INTV": 1.0, "PERIODIC": "T", "MinDepth": 0.01,
             "FIELD_IO_TYPE": "BINARY", "NumberStations": 3, "STATIONS_FILE": os.path.join(d, "stations.txt"),
             "PLOT_INTV_STATION": 1.0, "StationOutputBuffer": 2}
    _write_input(d, extra)
    r = subprocess.run([_driver(fw), os.path.join(d, "input.txt")], capture_output=True, text=True, cwd=d,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    files = sorted(f for f in os.listdir(d) if f.startswith("eta_"))
    assert len(files) >= 3
    etas = [np.fromfile(os.path.join(d, f), dtype=np.float64).reshape(16, 24).T for f in files]
    i0 = int(20.0 / 2.0) + 1
    I = np.arange(1, 25)
    wet = np.where(I >= i0, 3.0 - 0.2 * (I - i0) * 2.0, 3.0) > 0.0
    assert np.all(etas[0][wet, :] == 0.0)  # still water; dry land holds MinDepth - h
    assert np.abs(etas[-1][wet, :]).max() > 1e-4
    assert sorted(f for f in os.listdir(d) if f.startswith("sta_")) == ["sta_0001", "sta_0002"]
    rows = np.array([[float(line[:21])] + [float(line[21 + 16 * k:37 + 16 * k]) for k in range(3)]
                     for line in open(os.path.join(d, "sta_0001"))])
    times = np.loadtxt(os.path.join(d, "time_dt.out"), ndmin=2)[:, 0]
    assert rows.shape[0] == len(files)  # one sample per output (same interval), none dropped
    assert np.allclose(rows[:, 0], times, rtol=1e-9)
    for k, e in enumerate(etas):
        assert abs(rows[k, 1] - e[5, 4]) <= 1e-5 * max(abs(e[5, 4]), 1e-3)
    # station 2 sits at x = 24 m on dry land: zeros
    rows2 = np.loadtxt(os.path.join(d, "sta_0002"), ndmin=2)
    assert np.all(rows2[:, 1:] == 0.0)


@pytest.mark.gpu
def test_get_points_equals_fields(fw):
    import ctypes
    p, depth, _ = fw.cases.planar_beach(Mglob=40, Nglob=24, seed=21)
    for prec in ("FP64", "MIXED"):
        s = fw.Solver(fw.with_defaults(p), precision=prec)
        s.init(depth)
        s.step(5)
        I = np.array([1, 4, 20, 46, 33], dtype=np.int32)
        J = np.array([1, 4, 12, 30, 7], dtype=np.int32)
        for name in ("Eta", "U", "MASK", "P"):
            out = np.zeros(5)
            rc = s.L.fw_get_points(s.ctx, name.encode(), 5, I.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   J.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            assert rc == 0
            full = s.get(name)
            assert np.array_equal(out, full[I - 1, J - 1].astype(float)), name
        bad = np.array([47], dtype=np.int32)  # beyond Mloc = 46
        out = np.zeros(1)
        rc = s.L.fw_get_points(s.ctx, b"Eta", 1, bad.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                               J[:1].ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                               out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert rc == -3
        s.close()


def _run_driver(fw, d, extra):
    _write_input(d, extra)
    r = subprocess.run([_driver(fw), os.path.join(d, "input.txt")], capture_output=True, text=True, cwd=d,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


_SLOPE = {"DEPTH_TYPE": "SLOPE", "DEPTH_FLAT": 3.0, "SLP": 0.2, "Xslp": 20.0, "WAVEMAKER": "WK_REG",
          "AMP_WK": 0.05, "Tperiod": 3.0, "DEP_WK": 3.0, "Xc_WK": 10.0, "Time_ramp": 1.0, "PERIODIC": "T",
          "MinDepth": 0.01, "FIELD_IO_TYPE": "BINARY"}


@pytest.mark.gpu
def test_driver_hot_start_continues_the_run_exactly(fw, tmp_path):
    """HOTSTART_INTV writes exact checkpoints (fw_checkpoint); a run with
    HOT_START from one of them writes the same files, byte for byte, as the
    uninterrupted run from that point on: fields, time_dt.out and station
    rows."""
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    os.makedirs(a)
    os.makedirs(b)
    for d in (a, b):
        with open(os.path.join(d, "stations.txt"), "w") as f:
            f.write("6 5\n12 9\n")
    common = dict(_SLOPE, TOTAL_TIME=4.0, PLOT_INTV=0.5, NumberStations=2, PLOT_INTV_STATION=0.25,
                  StationOutputBuffer=3, PRECISION="MIXED")
    _run_driver(fw, a, dict(common, STATIONS_FILE=os.path.join(a, "stations.txt"), HOTSTART_INTV=1.5))
    assert sorted(f for f in os.listdir(a) if f.startswith("hotstart_")) == [
        "hotstart_00001", "hotstart_00001.host", "hotstart_00002", "hotstart_00002.host"]
    ck = os.path.join(a, "hotstart_00001")
    n_before = int(open(ck + ".host").read().split()[0])  # files written before the checkpoint
    _run_driver(fw, b, dict(common, STATIONS_FILE=os.path.join(b, "stations.txt"), HOT_START="T",
                            HOTSTART_FILE=ck))
    fa = sorted(f for f in os.listdir(a) if f.startswith(("eta_", "u_", "v_", "mask_")))
    fb = sorted(f for f in os.listdir(b) if f.startswith(("eta_", "u_", "v_", "mask_")))
    assert fb == [f for f in fa if int(f.split("_")[1]) > n_before] and len(fb) >= 8
    for f in fb:
        assert open(os.path.join(a, f), "rb").read() == open(os.path.join(b, f), "rb").read(), f
    ta = open(os.path.join(a, "time_dt.out")).read().splitlines()
    tb = open(os.path.join(b, "time_dt.out")).read().splitlines()
    assert tb == ta[n_before:]
    for k in ("sta_0001", "sta_0002"):
        ra = open(os.path.join(a, k)).read().splitlines()
        rb = open(os.path.join(b, k)).read().splitlines()
        assert len(rb) >= 4 and ra[len(ra) - len(rb):] == rb
    # the restored run's next checkpoint falls on the same pass with the
    # same counters
    _run_driver(fw, b, dict(common, STATIONS_FILE=os.path.join(b, "stations.txt"), HOT_START="T",
                            HOTSTART_FILE=ck, HOTSTART_INTV=1.5))
    for f in ("hotstart_00002.host",):
        assert open(os.path.join(a, f)).read() == open(os.path.join(b, f)).read()
    assert os.path.getsize(os.path.join(a, "hotstart_00002")) == os.path.getsize(os.path.join(b, "hotstart_00002"))


@pytest.mark.gpu
def test_driver_ini_uvz_hot_start_time(fw, tmp_path):
    """INI_UVZ (init.F:1283-1386): eta, u, v from ETA_FILE, U_FILE, V_FILE
    (list-directed rows of Mglob values) and TIME = HotStartTime
    (main.F:188-190): the run equals the Solver initialised with the same
    state and TIME; without V_FILE u and v start at zero."""
    d = str(tmp_path)
    rng = np.random.default_rng(3)
    I = np.arange(1, 25)
    i0 = int(20.0 / 2.0) + 1
    h = np.where(I >= i0, 3.0 - 0.2 * (I - i0) * 2.0, 3.0)
    depth = np.asfortranarray(np.repeat(h[:, None], 16, axis=1))
    wet = depth > 0.5
    eta = np.where(wet, 0.02 * rng.standard_normal((24, 16)), 0.0)
    u = np.where(wet, 0.05 * rng.standard_normal((24, 16)), 0.0)
    v = np.where(wet, 0.05 * rng.standard_normal((24, 16)), 0.0)
    for name, arr in (("eta0.txt", eta), ("u0.txt", u), ("v0.txt", v)):
        with open(os.path.join(d, name), "w") as f:
            for j in range(16):
                f.write(" ".join("%.17e" % x for x in arr[:, j]) + "\n")
    t0 = 7.25
    keys = _write_input(d, dict(_SLOPE, TOTAL_TIME=t0 + 1.0, PLOT_INTV=0.5, INI_UVZ="T", HotStartTime=t0,
                                ETA_FILE=os.path.join(d, "eta0.txt"), U_FILE=os.path.join(d, "u0.txt"),
                                V_FILE=os.path.join(d, "v0.txt")))
    r = subprocess.run([_driver(fw), os.path.join(d, "input.txt")], capture_output=True, text=True, cwd=d,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    times = np.loadtxt(os.path.join(d, "time_dt.out"), ndmin=2)
    assert times[0, 0] == t0
    files = sorted(f for f in os.listdir(d) if f.startswith("eta_"))
    first = np.fromfile(os.path.join(d, files[0]), dtype=np.float64).reshape(16, 24).T
    kept = eta >= -depth  # elsewhere dry: eta = -MinDepth - depth (init.F:1000-1014)
    assert np.array_equal(first[kept], eta[kept]) and np.all(first[~kept] == -0.01 - depth[~kept])
    p = {k: v for k, v in keys.items() if k not in ("RESULT_FOLDER", "FIELD_IO_TYPE", "INI_UVZ", "HotStartTime",
                                                     "ETA_FILE", "U_FILE", "V_FILE", "DEPTH_TYPE", "DEPTH_FLAT",
                                                     "SLP", "Xslp")}
    p["PERIODIC"] = True
    s = fw.Solver(fw.with_defaults(p), precision="FP64")
    s.init(depth, np.asfortranarray(eta), np.asfortranarray(u), np.asfortranarray(v))
    s.set_scalar("TIME", t0)
    while s.scalar("TIME") < times[-1, 0] * (1.0 - 1e-12):
        s.step(1)
    last = np.fromfile(os.path.join(d, files[-1]), dtype=np.float64).reshape(16, 24).T
    assert np.array_equal(last, s.get("Eta")[3:-3, 3:-3])
    s.close()
    # no V_FILE: u and v start at zero
    os.remove(os.path.join(d, "time_dt.out"))
    _write_input(d, dict(_SLOPE, TOTAL_TIME=t0 + 0.1, PLOT_INTV=0.5, INI_UVZ="T", HotStartTime=t0,
                         ETA_FILE=os.path.join(d, "eta0.txt"), U_FILE=os.path.join(d, "u0.txt")))
    r = subprocess.run([_driver(fw), os.path.join(d, "input.txt")], capture_output=True, text=True, cwd=d,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    u1 = np.fromfile(os.path.join(d, "u_00001"), dtype=np.float64).reshape(16, 24).T
    assert np.all(u1 == 0.0)


@pytest.mark.gpu
def test_driver_preview_mean_files(fw, tmp_path):
    """PREVIEW_MEAN (io.F:4630-4736): at the end of every CALCULATE_MEAN
    interval the driver writes umean/ulagm, vmean/vlagm, etamean, Hrms/Havg/
    Hsig and the Radiation files numbered by interval; the last set equals
    the Solver's means after the same steps (binary, bit for bit)."""
    d = str(tmp_path)
    extra = dict(_SLOPE, TOTAL_TIME=3.2, PLOT_INTV=10.0, STEADY_TIME=0.0, T_INTV_mean=1.0, Umean="T",
                 Vmean="T", ETAmean="T", WaveHeight="T", Radiation="T", Cd=0.003)
    keys = _run_driver(fw, d, extra)
    n = len([f for f in os.listdir(d) if f.startswith("etamean_")])
    assert n == 3
    for stem in ("umean", "ulagm", "vmean", "vlagm", "Hrms", "Havg", "Hsig", "Sxx", "Sxy", "Syy", "DxSxx",
                 "DySxy", "DySyy", "DxSxy", "PgrdX", "PgrdY", "DxUUH", "DyUVH", "DyVVH", "DxUVH", "FRCX", "FRCY",
                 "BrkDissX", "BrkDissY"):
        assert os.path.exists(os.path.join(d, "%s_%05d" % (stem, n))), stem
    p = {k: v for k, v in _SLOPE.items() if k not in ("FIELD_IO_TYPE", "DEPTH_TYPE", "DEPTH_FLAT", "SLP", "Xslp")}
    p.update({"Mglob": 24, "Nglob": 16, "DX": 2.0, "DY": 2.0, "PERIODIC": True, "STEADY_TIME": 0.0,
              "T_INTV_mean": 1.0, "OUT_Radiation": True, "OUT_Umean": True, "Cd": 0.003})
    i0 = int(20.0 / 2.0) + 1
    I = np.arange(1, 25)
    depth = np.asfortranarray(np.repeat(np.where(I >= i0, 3.0 - 0.2 * (I - i0) * 2.0, 3.0)[:, None], 16, axis=1))
    s = fw.Solver(fw.with_defaults(p), precision="FP64")
    s.init(depth)
    while s.scalar("TIME") < 3.2:
        s.step(1)
    assert s.scalar("ICOUNT_MEAN") == n

    def rd(stem):
        return np.fromfile(os.path.join(d, "%s_%05d" % (stem, n)), dtype=np.float64).reshape(16, 24).T

    def cur(name):
        return s.get(name)[3:-3, 3:-3]

    for stem, name in (("etamean", "ETAmean"), ("umean", "Umean"), ("Hsig", "SigWaveHeight"), ("Sxy", "UVmean"),
                       ("DxSxx", "DxSxx"), ("PgrdX", "PgrdX"), ("DyVVH", "DyVVH"), ("FRCX", "FRCXmean"),
                       ("BrkDissX", "BreakDissX")):
        assert np.array_equal(rd(stem), cur(name)), stem
    c49 = float(np.float32(0.5) * np.float32(9.8))
    assert np.array_equal(rd("Sxx"), cur("UUmean") - cur("WWmean") + c49 * cur("ETA2mean"))
    hm = np.maximum(cur("Depth") + cur("ETAmean"), 0.1)
    assert np.array_equal(rd("ulagm"), cur("P_mean") / hm)
    assert np.abs(rd("DxSxx")).max() > 0 and np.abs(rd("FRCX")).max() > 0
    s.close()
