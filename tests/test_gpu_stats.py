"""Statistics of the step: MAX_MIN_PROPERTY (misc.F:307-383) and
MIXING_STUFF / CALCULATE_MEAN (mixing.F:53-305) on the GPU against the
oracle.

FP64: whole steps with every switch on and several averaging intervals; the
fields follow the state, which agrees with the oracle to ~1e-9 after these
steps, so the statistics are checked at 1e-8 of their scale; the wave
heights, which hinge on discrete zero-up-crossing events, cell by cell.  Mixed: the float sums are Kahan-compensated; the
time-mean eta over a long interval is checked against the FP64 solver's.
"""
import numpy as np
import pytest

from helpers import G, interior, make_pair

pytestmark = pytest.mark.gpu

# fields that follow the state continuously
STATS = ("HeightMax", "HeightMin", "VelocityMax", "MomentumFluxMax", "ETAmean", "Umean", "Vmean",
         "ETA2mean", "SigWaveHeight")
# fields driven by discrete zero-up-crossing events: a cell where Eta passes
# ETAmean within rounding of a step boundary may see its crossing one step
# earlier or later, so these are compared cell by cell and a few cells
# (at most 0.1 %) may differ
EVENTS = ("WaveHeightAve", "WaveHeightRMS", "Emax", "Emin", "Num_Zero_Up")


def _stat_params(fw, Mglob, Nglob, seed, t_intv):
    p, depth, _ = fw.cases.planar_beach(Mglob=Mglob, Nglob=Nglob, seed=seed)
    p.update({"OUT_Hmax": True, "OUT_Hmin": True, "OUT_Umax": True, "OUT_MFmax": True,
              "STEADY_TIME": 0.0, "T_INTV_mean": t_intv})
    return p, depth


def test_statistics_fp64_parity(fw, oracle_mod):
    p, depth = _stat_params(fw, 64, 48, 7, 0.5)
    s, o = make_pair(fw, oracle_mod, p, depth)
    for _ in range(45):
        s.step(1)
        o.step()
    assert abs(s.scalar("T_sum") - o.scalar("T_sum")) <= 1e-9 * max(1.0, abs(o.scalar("T_sum")))
    assert s.scalar("TIME") > 2.0 * 0.5  # at least two intervals ended
    for name in STATS:
        a, b = s.get(name), o[name]
        scale = max(float(np.abs(b).max()), 1e-3)
        e = float(np.abs(a - b).max()) / scale
        assert e <= 1e-8, "%s: %.3e" % (name, e)
    assert np.abs(o["ETAmean"]).max() > 0.0 and o["Num_Zero_Up"].max() >= 2
    for name in EVENTS:
        a, b = s.get(name), np.asarray(o[name], dtype=float)
        scale = max(float(np.abs(b).max()), 1e-3)
        bad = np.abs(a - b) > 1e-8 * scale
        assert bad.mean() <= 1e-3, "%s: %d of %d cells differ" % (name, int(bad.sum()), bad.size)


def test_statistics_mixed_against_fp64(fw):
    """300 steps (about 15 s) with 6 s averaging intervals: ETAmean of the
    second interval and the running maximum, mixed against FP64."""
    p, depth = _stat_params(fw, 96, 64, 9, 6.0)
    res = {}
    for prec in ("FP64", "MIXED"):
        s = fw.Solver(fw.with_defaults(p), precision=prec)
        s.init(depth)
        s.step(300)
        res[prec] = (interior(s.get("ETAmean")), interior(s.get("HeightMax")), s.scalar("TIME"))
        s.close()
    em, hm, tm = res["MIXED"]
    ed, hd, td = res["FP64"]
    assert td > 12.0 and abs(tm - td) <= 1e-3 * td
    assert np.abs(ed).max() > 0.0
    assert float(np.sqrt(np.mean((em - ed) ** 2))) <= 1e-4
    assert float(np.abs(hm - hd).max()) <= 5e-3
