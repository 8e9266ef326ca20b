"""Known answers for the oracle's statistics (MIXING_STUFF / CALCULATE_MEAN,
mixing.F:53-305; MAX_MIN_PROPERTY, misc.F:307-383), from a sampled sine
wave whose mean, variance, up-crossings and crest-to-trough heights are
known in closed form.  CPU only."""
import math

import numpy as np
import pytest

A = 0.3       # amplitude (m)
T = 8.0       # period (s)
NPER = 64     # samples per period
G = 3


def _oracle(oracle_mod, params):
    p = {"Mglob": 4, "Nglob": 4, "DX": 1.0, "DY": 1.0, "DISPERSION": False}
    p.update(params)
    o = oracle_mod.Oracle(p)
    o["Depth"][...] = 5.0
    o.init()
    return o


def _drive(o, nsteps, dt, phase_steps=0.5):
    """Set Eta0 (the previous Eta) and Eta = A sin(2 pi t / T) on every cell
    at t = (k + phase_steps) dt, TIME = t, then MIXING_STUFF."""
    eta_prev = None
    for k in range(nsteps):
        t = (k + phase_steps) * dt
        eta = A * math.sin(2.0 * math.pi * t / T)
        o["Eta0"][...] = eta if eta_prev is None else eta_prev
        o["Eta"][...] = eta
        o.set_scalar("DT", dt)
        o.set_scalar("TIME", t)
        o.call("mixing_stuff")
        eta_prev = eta


def test_mean_variance_and_wave_heights_of_a_sine(oracle_mod):
    dt = T / NPER
    nper = 4
    o = _oracle(oracle_mod, {"STEADY_TIME": 0.0, "T_INTV_mean": nper * T - 0.5 * dt})
    _drive(o, nper * NPER, dt)
    c = (slice(G, -G), slice(G, -G))
    # the interval ended on the last sample: means of whole periods
    assert np.allclose(o["ETAmean"][c], 0.0, atol=1e-12)
    assert np.allclose(o["Umean"][c], 0.0)
    assert np.allclose(o["ETA2mean"][c], A * A / 2.0, rtol=1e-12)
    c4 = float(np.float32(4.004))
    assert np.allclose(o["SigWaveHeight"][c], c4 * math.sqrt(A * A / 2.0), rtol=1e-12)
    # up-crossings at t = T, 2T, 3T (the samples start just after t = 0 and
    # end just before 4T); heights from the second crossing on are the
    # sampled crest-to-trough 2 A cos(pi / NPER)
    assert (o["Num_Zero_Up"][c] == nper - 1).all()
    # (the reference divides the sums by every crossing, the first included,
    # which adds no height: mixing.F:249-252, 291-294)
    h = 2.0 * A * math.cos(math.pi / NPER)
    n = nper - 1
    assert np.allclose(o["WaveHeightAve"][c], (n - 1) * h / n, rtol=1e-12)
    assert np.allclose(o["WaveHeightRMS"][c], math.sqrt((n - 1) * h * h / n), rtol=1e-12)
    assert o.scalar("T_sum") == pytest.approx(0.5 * dt, rel=1e-9)


def test_nothing_before_steady_time(oracle_mod):
    dt = T / NPER
    o = _oracle(oracle_mod, {"STEADY_TIME": 1.0e3, "T_INTV_mean": 2 * T})
    _drive(o, 3 * NPER, dt)
    assert o.scalar("T_sum") == 0.0
    assert not o["ETA2mean"].any() and not o["Num_Zero_Up"].any()


def test_running_extrema(oracle_mod):
    o = _oracle(oracle_mod, {})
    o.init()
    o["MASK"][...] = 1
    seq = [0.1, -0.2, 0.35, 0.05]
    for e in seq:
        o["Eta"][...] = e
        o["U"][...] = e
        o["V"][...] = 2 * e
        o["H"][...] = 5.0 + e
        o.call("max_min_property")
    assert np.allclose(o["HeightMax"], max(0.0, max(seq)))
    # HeightMin, VelocityMax, MomentumFluxMax stay off unless switched on
    assert not o["HeightMin"].any() and not o["VelocityMax"].any()
    o2 = _oracle(oracle_mod, {"OUT_Hmin": True, "OUT_Umax": True, "OUT_MFmax": True})
    o2["MASK"][...] = 1
    for e in seq:
        o2["Eta"][...] = e
        o2["U"][...] = e
        o2["V"][...] = 2 * e
        o2["H"][...] = 5.0 + e
        o2.call("max_min_property")
    assert np.allclose(o2["HeightMin"], min(0.0, min(seq)))
    assert np.allclose(o2["VelocityMax"], max(math.sqrt(5.0) * abs(e) for e in seq))
    assert np.allclose(o2["MomentumFluxMax"], max(5.0 * e * e * (5.0 + e) for e in seq))


def test_radiation_means_and_gradients(oracle_mod):
    """CALCULATE_MEAN's radiation part (mixing.F:156-219) on driven fields:
    with constant U_davg, Wsurf, P_center, BreakSourceX over one interval
    the means equal the inputs (UU about the previous, zero, U_davg_mean,
    weighed by the depth with the ETAmean each step sees),
    and the gradient fields are the centred differences of the means with
    the reference's default-REAL 9.80 and 0.5*9.80; FRCXmean carries Cd on
    the interior only."""
    o = _oracle(oracle_mod, {"Mglob": 8, "Nglob": 6, "STEADY_TIME": 0.0, "T_INTV_mean": 1.0})
    M, N = o["Eta"].shape
    rng = np.random.default_rng(5)
    ud = rng.uniform(0.1, 0.5, (M, N))
    ws = rng.uniform(-0.2, 0.2, (M, N))
    pc = rng.uniform(0.5, 1.5, (M, N))
    bx = rng.uniform(-1e-3, 1e-3, (M, N))
    eta = rng.uniform(-0.1, 0.1, (M, N))
    u = rng.uniform(-0.3, 0.3, (M, N))
    o["Cd"][...] = 0.002
    dt = 0.25
    for k in range(4):  # 4 x 0.25 s: the interval ends at the fourth step
        o["U_davg"][...] = ud
        o["V_davg"][...] = 0.0
        o["P_center"][...] = pc
        o["Q_center"][...] = 0.0
        o["Wsurf"][...] = ws
        o["BreakSourceX"][...] = bx
        o["Eta"][...] = eta
        o["Eta0"][...] = eta
        o["U"][...] = u
        o["V"][...] = 0.0
        o.set_scalar("DT", dt)
        o.set_scalar("TIME", (k + 1) * dt)
        o.call("mixing_stuff")
    assert np.allclose(o["U_davg_mean"], ud, rtol=1e-12)
    assert np.allclose(o["P_mean"], pc, rtol=1e-12)
    assert np.allclose(o["BreakDissX"], bx, rtol=1e-12, atol=1e-18)
    em = o["ETAmean"]
    assert np.allclose(em, eta, rtol=1e-12, atol=1e-15)
    # the first three steps weigh by Eta - ETAmean + Depth with the previous
    # interval's ETAmean (0), the last with the new one (= Eta), in the
    # reference's statement order (mixing.F:154-163)
    D = o["Depth"]
    hw = (3.0 * (eta + D) + D) / 4.0
    assert np.allclose(o["UUmean"], ud * ud * hw, rtol=1e-12)  # about the previous U_davg_mean, 0
    assert np.allclose(o["WWmean"], 0.25 * ws * ws * hw, rtol=1e-12)
    inner = (slice(G, -G), slice(G, -G))
    frcx = u * np.abs(u)
    assert np.allclose(o["FRCXmean"][inner], (frcx * 0.002)[inner], rtol=1e-12)
    ring = np.ones((M, N), bool)
    ring[inner] = False
    assert np.allclose(o["FRCXmean"][ring], frcx[ring], rtol=1e-12)
    dx = 1.0
    g49 = float(np.float32(0.5) * np.float32(9.80))
    g98 = float(np.float32(9.80))
    uu, wwm, e2 = o["UUmean"], o["WWmean"], o["ETA2mean"]
    want = ((uu[2:, 1:-1] - uu[:-2, 1:-1]) / 2.0 / dx - (wwm[2:, 1:-1] - wwm[:-2, 1:-1]) / 2.0 / dx
            + g49 * (e2[2:, 1:-1] - e2[:-2, 1:-1]) / 2.0 / dx)
    assert np.allclose(o["DxSxx"][inner], want[G - 1:-(G - 1), G - 1:-(G - 1)], rtol=1e-12, atol=1e-18)
    pg = g98 * (o["Depth"] + em)[1:-1, 1:-1] * (em[2:, 1:-1] - em[:-2, 1:-1]) / 2.0 / dx
    assert np.allclose(o["PgrdX"][inner], pg[G - 1:-(G - 1), G - 1:-(G - 1)], rtol=1e-12, atol=1e-18)
    hm = np.maximum(o["Depth"] + em, 0.1)
    pm = o["P_mean"]
    duu = (pm[2:, 1:-1] ** 2 / hm[2:, 1:-1] - pm[:-2, 1:-1] ** 2 / hm[:-2, 1:-1]) / 2.0 / dx
    assert np.allclose(o["DxUUH"][inner], duu[G - 1:-(G - 1), G - 1:-(G - 1)], rtol=1e-12)
    # the sums restart
    assert np.all(o["UUsum"] == 0.0) and np.all(o["P_sum"] == 0.0)
