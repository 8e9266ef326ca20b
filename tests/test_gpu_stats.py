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


# CALCULATE_MEAN's radiation-stress, momentum-flux and breaking-dissipation
# part (mixing.F:156-219) with the last stage's inputs (etauv_solver.F:94-101,
# 247; sources.F:428-456) and their exchange (bc.F:438-443)
RAD_STEP = ("P_center", "Q_center", "U_davg", "V_davg", "Wsurf", "BreakSourceX", "BreakSourceY")
RAD_MEANS = ("U_davg_mean", "V_davg_mean", "P_mean", "Q_mean", "UUmean", "UVmean", "VVmean", "WWmean",
             "FRCXmean", "FRCYmean", "BreakDissX", "BreakDissY")
RAD_GRAD = ("DxSxx", "DySxy", "DySyy", "DxSxy", "PgrdX", "PgrdY", "DxUUH", "DyUVH", "DyVVH", "DxUVH")


def _rad_params(fw, Mglob, Nglob, seed, t_intv, periodic=True):
    p, depth = _stat_params(fw, Mglob, Nglob, seed, t_intv)
    p.update({"OUT_Radiation": True, "PERIODIC": periodic, "Cd": 0.002})
    return p, depth


@pytest.mark.parametrize("periodic", [True, False])
def test_radiation_fp64_parity(fw, oracle_mod, periodic):
    p, depth = _rad_params(fw, 64, 48, 7, 0.5, periodic)
    s, o = make_pair(fw, oracle_mod, p, depth)
    for _ in range(45):
        s.step(1)
        o.step()
    assert s.scalar("ICOUNT_MEAN") >= 2  # at least two intervals ended
    for name in RAD_STEP:
        a, b = s.get(name), o[name]
        scale = max(float(np.abs(b).max()), 1e-6)
        e = float(np.abs(a - b).max()) / scale
        assert e <= 1e-9, "%s: %.3e" % (name, e)
    for name in RAD_MEANS + RAD_GRAD:
        a, b = s.get(name), o[name]
        scale = float(np.abs(b).max())
        assert scale > 0.0 or name.startswith("BreakDiss"), name
        e = float(np.abs(a - b).max()) / max(scale, 1e-12)
        assert e <= 1e-8, "%s: %.3e" % (name, e)
    s.close()


def test_radiation_mixed_against_fp64(fw):
    """Mixed against FP64 after 300 steps with 6 s intervals: the means of
    the second interval to a few 1e-3 of their scale (the float sums are
    Kahan-compensated; the flows differ at the stated eta error)."""
    p, depth = _rad_params(fw, 96, 64, 9, 6.0)
    res = {}
    for prec in ("FP64", "MIXED"):
        s = fw.Solver(fw.with_defaults(p), precision=prec)
        s.init(depth)
        s.step(300)
        res[prec] = {n: interior(s.get(n)) for n in RAD_MEANS[:10] + ("DxSxx", "PgrdX")}
        assert s.scalar("ICOUNT_MEAN") >= 2
        s.close()
    for n, d in res["FP64"].items():
        m = res["MIXED"][n]
        scale = float(np.abs(d).max())
        assert scale > 0.0, n
        rms = float(np.sqrt(np.mean((m - d) ** 2))) / scale
        assert rms <= 5e-3, "%s: %.3e" % (n, rms)


def test_radiation_fields_absent_when_off(fw):
    p, depth = _stat_params(fw, 32, 24, 1, 0.5)
    s = fw.Solver(fw.with_defaults(p), precision="MIXED")
    s.init(depth)
    s.step(4)
    for n in ("UUmean", "DxSxx", "Wsurf"):
        with pytest.raises(fw.FwError):
            s.get(n)
    s.close()
