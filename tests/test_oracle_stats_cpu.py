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
