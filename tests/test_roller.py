"""Roller flux and undertow of BREAKING (breaker.F:316-339), switched on by
the ROLLER / UNDERTOW output keys: the GPU against the oracle on a barred
beach whose waves break on the bar and the beach.

A cell's roller is written when it is breaking (0 < AGE < T_brk and ETAt
above Cbrk2 sqrt(g H)) and keeps its value otherwise, so the fields record
the last breaking event of every cell.  Breaking onsets are threshold
events: a cell where ETAt passes the threshold within rounding of a step may
start one step earlier or later on the GPU than in the oracle, so the fields
are compared cell by cell and a few cells (at most 1 %) may differ.
"""
import numpy as np
import pytest

from helpers import G, make_pair

pytestmark = pytest.mark.gpu

# with the breaking-dissipation means of CALCULATE_MEAN (mixing.F:166-180),
# which sum BreakSourceX/Y of the last stage
FIELDS = ("ROLLER_FLUX", "UNDERTOW_U", "UNDERTOW_V", "BreakDissX", "BreakDissY", "BreakSourceX")


def _case(fw):
    p, d, ph, _ = fw.cases.barred_beach(480, 64, 1.0, seed=4, wk_from_shore=120.0)
    p.update({"ROLLER": True, "UNDERTOW": True, "STEADY_TIME": 0.0, "T_INTV_mean": 4.0, "OUT_Radiation": True})
    return p, d, ph


def test_roller_and_undertow_fp64_parity(fw, oracle_mod):
    p, d, ph = _case(fw)
    s, o = make_pair(fw, oracle_mod, p, d, phases=ph)
    for _ in range(520):
        assert s.step(1) == 0
        assert o.step() == 0
    rf = o["ROLLER_FLUX"][G:-G, G:-G]
    assert (rf != 0).sum() >= 20  # breaking has started
    assert np.abs(o["ETAmean"]).max() > 0  # the roller sees a time-mean eta
    for name in FIELDS:
        a, b = s.get(name)[G:-G, G:-G], o[name][G:-G, G:-G]
        scale = float(np.abs(b).max())
        assert scale > 0, name
        bad = np.abs(a - b) > 1e-8 * scale
        assert bad.mean() <= 0.01, "%s: %d of %d cells differ" % (name, int(bad.sum()), bad.size)
        same = ~bad
        assert float(np.abs(a - b)[same].max()) <= 1e-8 * scale
    # the undertow points against the propagation direction: |undertow| = |roller|
    u, v = s.get("UNDERTOW_U")[G:-G, G:-G], s.get("UNDERTOW_V")[G:-G, G:-G]
    r = s.get("ROLLER_FLUX")[G:-G, G:-G]
    assert np.allclose(np.hypot(u, v), np.abs(r), rtol=1e-9, atol=1e-14)
    s.close()


def test_roller_mixed_runs_and_fields_are_absent_when_off(fw):
    p, d, ph = _case(fw)
    s = fw.Solver(fw.with_defaults(p), precision="MIXED")
    s.init(d, phases=ph)
    assert s.step(520) == 0
    r = s.get("ROLLER_FLUX")[G:-G, G:-G]
    assert np.isfinite(r).all() and (r != 0).sum() >= 20
    s.close()
    q = dict(p)
    q["ROLLER"] = q["UNDERTOW"] = False
    s = fw.Solver(fw.with_defaults(q), precision="MIXED")
    s.init(d, phases=ph)
    with pytest.raises(fw.FwError):
        s.get("ROLLER_FLUX")
    s.close()
