"""GPU parity with the CPU oracle, unit by unit and over whole steps.

FP64: the kernels keep the reference's operation order without fused
multiply-adds and solve the tridiagonal systems with the reference's Thomas
recurrence, so they differ from the oracle only where CUDA's libm (exp, sin,
cos, tanh, atan2 in the wavemaker, breaking and Froude cap) rounds its last
bit differently from glibc: every field within 1e-11 of its scale per unit,
MASK and MASK9 bit-exact.  Mixed precision: eta within 1e-4 m of the FP64 oracle after the
stated steps, MASK mismatches counted.
"""
import numpy as np
import pytest

from helpers import G, interior, make_pair, maxrel, sloped_beach

pytestmark = pytest.mark.gpu

TOL = 1e-11
ATOL = 1e-14  # absolute floor for values that are exact zeros in one of the two


def _regions(s):
    M, N = s.Mloc, s.Nloc
    return {
        "int": (slice(G, M - G), slice(G, N - G)),
        "ring": (slice(G - 1, M - G + 1), slice(G - 1, N - G + 1)),
        "all": (slice(0, M), slice(0, N)),
        "xf": (slice(G, M - G + 1), slice(G, N - G)),
        "yf": (slice(G, M - G), slice(G, N - G + 1)),
    }


def _cmp(s, o, name, region, tol=TOL, oname=None, oval=None, exclude=None):
    r = _regions(s)[region]
    a = s.get(name)
    b = o[oname or name] if oval is None else oval
    a, b = np.array(a[r], dtype=float), np.array(b[r], dtype=float)
    if exclude is not None:
        a[exclude[r]] = 0.0
        b[exclude[r]] = 0.0
    e = float(np.abs(a - b).max()) / (max(float(np.abs(b).max()), 1e-30) + ATOL / tol)
    if not e <= tol:
        k = np.unravel_index(np.argmax(np.abs(a - b)), a.shape)
        raise AssertionError("%s (%s): rel err %.3e, max|ref| %.3e, worst at %s (+region offset) gpu %.17g ref %.17g"
                             % (name, region, e, np.abs(b).max(), k, a[k], b[k]))
    return e


def _corners(s):
    m = np.zeros((s.Mloc, s.Nloc), dtype=bool)
    for a in (slice(0, G), slice(s.Mloc - G, s.Mloc)):
        for b in (slice(0, G), slice(s.Nloc - G, s.Nloc)):
            m[a, b] = True
    return m


def _unit_pipeline(fw, oracle_mod, params, depth, state, nstages=6, phases=None):
    s, o = make_pair(fw, oracle_mod, params, depth, state, phases)
    per = bool(fw.with_defaults(params)["PERIODIC"])
    corners = _corners(s) if per else None
    for name in ("Depth", "H", "Eta", "Ubar", "Vbar", "HU", "HV", "SPONGE"):
        _cmp(s, o, name, "all")
    for name in ("Depthx", "Depthy"):
        r = "xf" if name == "Depthx" else "yf"
        a, b = s.get(name), o[name]
        assert maxrel(a, b) <= TOL, name
    assert np.array_equal(s.get("MASK"), o["MASK"])
    assert np.array_equal(s.get("MASK9"), o["MASK9"])
    for k in ("ilo", "ihi", "jlo", "jhi"):
        assert s.scalar(k) == o.scalar(k), k
    for k in ("Width_WK", "EtaBlowVal"):
        assert abs(s.scalar(k) - o.scalar(k)) <= 1e-12 * max(1.0, abs(o.scalar(k))), k
    stage = 0
    for step in range(nstages // 3 + 1):
        s.begin_step()
        o.begin_step()
        assert abs(s.scalar("DT") - o.scalar("DT")) <= 1e-12 * o.scalar("DT")
        assert abs(s.scalar("TIME") - o.scalar("TIME")) <= 1e-12 * o.scalar("TIME")
        for name in ("U", "V", "HU", "HV", "Eta", "U0", "V0", "Eta0", "Ubar0", "Vbar0"):
            _cmp(s, o, name, "all")
        for ist in (1, 2, 3):
            if stage >= nstages:
                return s, o
            stage += 1
            s.cal_dispersion()
            o.call("cal_dispersion")
            _cmp(s, o, "U4", "all", exclude=corners)
            _cmp(s, o, "V4", "all", exclude=corners)
            _cmp(s, o, "U1p", "int")
            _cmp(s, o, "V1p", "int")
            _cmp(s, o, "Udisp", "int", oval=(o["U1pp"] + o["U2"]) + o["U3"], tol=1e-8)
            _cmp(s, o, "Vdisp", "int", oval=(o["V1pp"] + o["V2"]) + o["V3"], tol=1e-8)
            _cmp(s, o, "ETAx", "ring")
            _cmp(s, o, "ETAy", "ring")
            _cmp(s, o, "ETAT", "ring")
            s.fluxes()
            o.call("fluxes")
            for name in ("P", "Fx", "Gx"):
                _cmp(s, o, name, "xf")
            for name in ("Q", "Fy", "Gy"):
                _cmp(s, o, name, "yf")
            s.source_terms()
            o.call("source_terms")
            _cmp(s, o, "SourceX", "int", tol=1e-8)
            _cmp(s, o, "SourceY", "int", tol=1e-8)
            _cmp(s, o, "WaveMaker_Mass", "int")
            s.estimate_huv(ist)
            o.call("estimate_huv", ist)
            for name in ("Eta", "Ubar", "Vbar", "U", "V", "HU", "HV"):
                _cmp(s, o, name, "int", tol=1e-8)
            _cmp(s, o, "H", "all", tol=1e-8)
            s.update_mask()
            o.call("update_mask")
            assert np.array_equal(s.get("MASK"), o["MASK"]), "MASK after UPDATE_MASK"
            assert np.array_equal(s.get("MASK9"), o["MASK9"]), "MASK9 after UPDATE_MASK"
            assert maxrel(s.get("Depthx"), o["Depthx"]) <= TOL
            assert maxrel(s.get("Depthy"), o["Depthy"]) <= TOL
            s.wave_breaking()
            o.call("wave_breaking")
            _cmp(s, o, "AGE", "ring")
            _cmp(s, o, "nu_break", "ring", tol=1e-8)
            s.exchange()
            o.call("exchange")
            if fw.with_defaults(params)["DIRECT_SPONGE"]:
                s.sponge_damping()
                o.call("sponge_damping")
            for name in ("Eta", "U", "V", "HU", "HV", "AGE", "nu_break"):
                _cmp(s, o, name, "all", tol=1e-8)
            assert np.array_equal(s.get("MASK"), o["MASK"]), "MASK after EXCHANGE"
            a, b = s.get("P"), o["P"]
            assert maxrel(a, b) <= 1e-8, "P after EXCHANGE"
            a, b = s.get("Q"), o["Q"]
            assert maxrel(a, b) <= 1e-8, "Q after EXCHANGE"
    return s, o


def test_units_periodic_planar_beach(fw, oracle_mod):
    p, depth, _ = fw.cases.planar_beach(Mglob=64, Nglob=40, seed=11)
    state = fw.cases.random_state(64, 40, seed=12, eta_amp=0.1, u_amp=0.2)
    _unit_pipeline(fw, oracle_mod, p, depth, state, nstages=6)


def test_units_walls_shoreline_breaking(fw, oracle_mod):
    p, _, _ = fw.cases.planar_beach(Mglob=72, Nglob=36, seed=21)
    p.update({"PERIODIC": False, "Xc_WK": 15.0, "DEP_WK": 1.5, "AMP_WK": 0.2, "Tperiod": 4.0,
              "Sponge_west_width": 8.0, "Cbrk1": 0.15, "Cbrk2": 0.05})
    depth = sloped_beach(72, 36, seed=22)
    state = fw.cases.random_state(72, 36, seed=23, eta_amp=0.25, u_amp=0.5, smooth=1.5)
    _unit_pipeline(fw, oracle_mod, p, depth, state, nstages=6)


def test_units_jonswap(fw, oracle_mod):
    p, depth, ph = fw.cases.shoal_jonswap(Mglob=80, Nglob=48, dx=4.0, seed=5)
    # shrink the geometry: 20 m flat water, JON_2D near the west wall
    depth = np.asfortranarray(np.full((80, 48), 20.0) - np.linspace(0, 22, 80)[:, None])
    p.update({"Nfreq": 8, "Ntheta": 5, "Xc_WK": 40.0, "Sponge_west_width": 16.0})
    ph = np.asfortranarray(ph[:8, :5])
    _unit_pipeline(fw, oracle_mod, p, depth, None, nstages=6, phases=ph)


@pytest.mark.parametrize("periodic", [True, False])
def test_whole_steps_fp64(fw, oracle_mod, periodic):
    p, depth, _ = fw.cases.planar_beach(Mglob=96, Nglob=50, seed=31)
    p.update({"PERIODIC": periodic, "Cbrk1": 0.2, "Cbrk2": 0.1})
    depth = sloped_beach(96, 50, h0=3.0, h1=-0.8, seed=32)
    state = fw.cases.random_state(96, 50, seed=33, eta_amp=0.2, u_amp=0.3)
    s, o = make_pair(fw, oracle_mod, p, depth, state)
    for k in range(5):
        s.step(4)
        for _ in range(4):
            o.step()
        assert np.array_equal(s.get("MASK"), o["MASK"]), "MASK after %d steps" % (4 * (k + 1))
        for name in ("Eta", "U", "V"):
            e = maxrel(interior(s.get(name)), interior(o[name]))
            assert e <= 1e-9, "%s after %d steps: %.3e" % (name, 4 * (k + 1), e)
    assert abs(s.scalar("TIME") - o.scalar("TIME")) <= 1e-10 * o.scalar("TIME")


def test_mixed_precision_error(fw, oracle_mod):
    p, depth, _ = fw.cases.planar_beach(Mglob=96, Nglob=50, seed=41)
    s, o = make_pair(fw, oracle_mod, p, depth, None, precision="MIXED")
    s.step(60)
    for _ in range(60):
        o.step()
    d = interior(s.get("Eta")) - interior(o["Eta"])
    rms = float(np.sqrt(np.mean(d * d)))
    assert rms <= 1e-4, "mixed eta rms %.3e" % rms


@pytest.mark.parametrize("periodic", [True, False])
def test_units_mixed_precision(fw, oracle_mod, periodic):
    """Mixed path, one step unit by unit against the FP64 oracle: float
    fields carry ~1e-7 relative rounding, the tridiagonal solve is FP64 on
    the constant factorisation; fields within 2e-4 of their scale."""
    p, depth, _ = fw.cases.planar_beach(Mglob=80, Nglob=64, seed=51)
    p.update({"PERIODIC": periodic})
    state = fw.cases.random_state(80, 64, seed=52, eta_amp=0.1, u_amp=0.2)
    s, o = make_pair(fw, oracle_mod, p, depth, state, precision="MIXED")
    s.begin_step()
    o.begin_step()
    for ist in (1, 2, 3):
        s.cal_dispersion()
        o.call("cal_dispersion")
        s.fluxes()
        o.call("fluxes")
        o.call("source_terms")
        s.estimate_huv(ist)
        o.call("estimate_huv", ist)
        for name in ("Eta", "Ubar", "Vbar", "U", "V"):
            e = maxrel(interior(s.get(name)), interior(o[name]), floor=1e-3)
            assert e <= 2e-4, "%s stage %d: %.3e" % (name, ist, e)
        s.update_mask()
        o.call("update_mask")
        s.wave_breaking()
        o.call("wave_breaking")
        s.exchange()
        o.call("exchange")
        s.sponge_damping()
        o.call("sponge_damping")


def test_mixed_vs_fp64_long_run(fw):
    """The 250 x 500 planar beach for 300 steps (about 21 s of waves):
    mixed precision (float fields, float line solve with one compensated
    refinement step) against the FP64 path, which matches the oracle: eta
    RMS over wet cells <= 1e-4 m, the error the mixed mode is specified to."""
    p, depth, _ = fw.cases.planar_beach(seed=7)
    d64 = fw.Solver(p, precision="FP64")
    d64.init(depth)
    mx = fw.Solver(p, precision="MIXED")
    mx.init(depth)
    d64.step(300)
    mx.step(300)
    e64, em = interior(d64.get("Eta")), interior(mx.get("Eta"))
    wet = interior(d64.get("MASK")) > 0
    rms = float(np.sqrt(np.mean((em - e64)[wet] ** 2)))
    assert rms <= 1e-4, "eta rms %.3e" % rms
    assert abs(d64.scalar("TIME") - mx.scalar("TIME")) < 1e-3 * d64.scalar("TIME")
