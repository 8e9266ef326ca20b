"""BREAKING's candidate sweep (breaker.F:182-224) when chains are long.

The sweep runs j outer, i inner; a candidate reads the new ages of the cells
before it and the old ages of the cells after it.  The kernel iterates in
parallel to the fixed point for BREAK_PASSES passes and finishes in one pass
ordered by level i + 2j.  Under the CFL limit a newly set age DT never
exceeds a cell's crossing time, so in a simulation chains stop after one
link; here DT = 1 s on 20 m of water (crossing time 1/14 s per cell) makes
every candidate carry the age on, and chains run across the grid.  Each
BREAK_PASSES value (0: the level-ordered pass alone; 1, 3, 8: both; a
million: passes alone) must give the oracle's sequential sweep bit for bit.
The mixed build's sweep breaks the same cells.  Whole mixed and FP64 steps
with the level-ordered pass alone give the same state as with the default.
"""
import numpy as np
import pytest

from helpers import G, interior, make_pair, maxrel, sloped_beach

pytestmark = pytest.mark.gpu


def _fields(Mloc, Nloc, t_brk, seed):
    """H, ETAT, ETAx, ETAy, AGE for one WAVE_BREAKING call: candidates almost
    everywhere, propagation directions mostly in the (0, 90) degree quadrant
    with patches of the other three, a few old breakers as sources."""
    rng = np.random.default_rng(seed)
    shape = (Mloc, Nloc)
    H = np.full(shape, 20.0)
    # sqrt(g H) = 14.0: Cbrk2 (0.35) gives 4.9 m/s, Cbrk1 (0.65) 9.1 m/s
    ETAT = 6.0 + 0.5 * rng.uniform(-1.0, 1.0, shape)
    r = rng.random(shape)
    ETAT[r < 0.002] = 10.0   # new breakers
    ETAT[r > 0.97] = 2.0     # not candidates
    quad = np.where(rng.random((Mloc // 12 + 1, Nloc // 12 + 1)) < 0.7, 0,
                    rng.integers(1, 4, (Mloc // 12 + 1, Nloc // 12 + 1)))
    quad = np.kron(quad, np.ones((12, 12), dtype=int))[:Mloc, :Nloc]
    ang = np.radians(quad * 90.0 + rng.uniform(5.0, 85.0, shape))
    # ANGLE = atan2(-ETAy, -ETAx): a gradient of 0.1 pointing against it
    ETAx = np.asfortranarray(-0.1 * np.cos(ang))
    ETAy = np.asfortranarray(-0.1 * np.sin(ang))
    AGE = np.zeros(shape)
    src = rng.choice(Mloc * Nloc, 12, replace=False)
    AGE.flat[src[:8]] = 0.5
    AGE.flat[src[8:]] = t_brk + 1.0   # restarts
    return {"H": H, "ETAT": np.asfortranarray(ETAT), "ETAx": ETAx, "ETAy": ETAy, "AGE": AGE}


def _ring(a):
    return a[G - 1:-(G - 1), G - 1:-(G - 1)]


@pytest.mark.parametrize("passes", [0, 1, 3, 8, 1000000])
def test_long_chains_match_oracle(fw, oracle_mod, passes):
    scipy_ndimage = pytest.importorskip("scipy.ndimage")
    params, depth, _ = fw.cases.planar_beach(Mglob=96, Nglob=64, seed=61)
    s, o = make_pair(fw, oracle_mod, params, depth)
    assert s.scalar("BREAK_PASSES") == 8
    fields = _fields(s.Mloc, s.Nloc, s.scalar("T_brk"), seed=62)
    for name, a in fields.items():
        s.set(name, a)
        o[name][:] = a
    s.set_scalar("DT", 1.0)
    o.set_scalar("DT", 1.0)
    s.set_scalar("BREAK_PASSES", passes)
    assert s.scalar("BREAK_PASSES") == passes
    s.wave_breaking()
    o.call("wave_breaking")
    age_o = _ring(o["AGE"])
    # the sweep set about the whole grid, far from any cell that was not a
    # candidate: a cell at chessboard distance d from every such breaker
    # needs d parallel passes, and the farthest lies beyond the default 8
    cand_set = (age_o == 1.0) & (_ring(fields["AGE"]) == 0.0) & (_ring(fields["ETAT"]) < 9.1)
    assert cand_set.sum() > 2000
    seeds = (age_o > 0.0) & ~cand_set
    dist = scipy_ndimage.distance_transform_cdt(~seeds, metric="chessboard")
    assert dist[cand_set].max() > 8
    assert np.array_equal(_ring(s.get("AGE")), age_o)
    assert maxrel(_ring(s.get("nu_break")), _ring(o["nu_break"])) <= 1e-12
    # the candidate counter is reset for the next call
    s.set("AGE", fields["AGE"])
    o["AGE"][:] = fields["AGE"]
    s.wave_breaking()
    o.call("wave_breaking")
    assert np.array_equal(_ring(s.get("AGE")), _ring(o["AGE"]))
    s.close()
    o.close()


@pytest.mark.parametrize("passes", [0, 8])
def test_long_chains_mixed(fw, oracle_mod, passes):
    """The same sweep in the mixed build: the float tests decide as the
    oracle's double ones on these well-separated values, so the same cells
    break, with ages equal to float rounding.  It also checks that a DT set
    from the host reaches the mixed build's float copy."""
    params, depth, _ = fw.cases.planar_beach(Mglob=96, Nglob=64, seed=61)
    s, o = make_pair(fw, oracle_mod, params, depth, precision="MIXED")
    fields = _fields(s.Mloc, s.Nloc, s.scalar("T_brk"), seed=62)
    for name, a in fields.items():
        s.set(name, a)
        o[name][:] = a
    s.set_scalar("DT", 1.0)
    o.set_scalar("DT", 1.0)
    s.set_scalar("BREAK_PASSES", passes)
    s.wave_breaking()
    o.call("wave_breaking")
    a, b = _ring(s.get("AGE")), _ring(o["AGE"])
    assert ((b == 1.0).sum()) > 2000
    assert np.array_equal(a > 0, b > 0)
    assert np.array_equal(a == 1.0, b == 1.0)
    assert np.allclose(a, b, rtol=1e-6, atol=0.0)
    s.close()
    o.close()


@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
def test_level_pass_alone_in_whole_steps(fw, oracle_mod, precision):
    """Graph-captured steps of a breaking beach with BREAK_PASSES = 0 give
    the state of the default bit for bit; FP64 also matches the oracle."""
    p, _, _ = fw.cases.planar_beach(Mglob=96, Nglob=50, seed=31)
    # low onset thresholds: breaking from the first steps, with candidates
    p.update({"PERIODIC": False, "Cbrk1": 0.03, "Cbrk2": 0.015})
    depth = sloped_beach(96, 50, h0=3.0, h1=-0.8, seed=32)
    state = fw.cases.random_state(96, 50, seed=33, eta_amp=0.2, u_amp=0.3)
    out = {}
    for passes in (8, 0):
        s, o = make_pair(fw, oracle_mod, p, depth, state, precision=precision)
        s.set_scalar("BREAK_PASSES", passes)
        s.step(12)
        out[passes] = {k: s.get(k) for k in ("Eta", "U", "V", "AGE", "nu_break")}
        if precision == "FP64" and passes == 0:
            for _ in range(12):
                o.step()
            assert np.array_equal(interior(s.get("AGE")), interior(o["AGE"]))
            for name in ("Eta", "U", "V"):
                assert maxrel(interior(s.get(name)), interior(o[name])) <= 1e-9, name
        s.close()
        o.close()
    assert (out[8]["AGE"] > 0).sum() > 100
    for k in out[8]:
        assert np.array_equal(out[8][k], out[0][k]), k
