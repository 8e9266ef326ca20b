"""Ensembles of independent runs (fw_ensemble_step): the member generator's
distribution (CPU), the run-up measure (CPU), and on the GPU that runs
stepped together equal the same runs stepped alone, bit for bit, with their
maximum run-up."""
import numpy as np
import pytest


def test_member_distribution(fw):
    m = fw.cases.ensemble_members(512, seed=1)
    cells = np.array([p["Mglob"] * p["Nglob"] for p, _, _ in m])
    assert len(m) == 512
    assert cells.min() >= 0.9 * 128 * 256 and cells.max() <= 1.1 * 1024 * 1024
    assert 1.2e8 <= cells.sum() <= 1.9e8  # about 1.5e8 cells in all
    for p, d, ph in m[:50]:
        assert 1.0 <= p["DX"] <= 4.0 and 0.5 <= p["Hmo"] <= 3.0 and 6.0 <= 1.0 / p["FreqPeak"] <= 14.0
        assert d.shape == (p["Mglob"], p["Nglob"]) and (d < 0).any() and d.max() <= 20.0
        assert ph.shape == (p["Nfreq"], p["Ntheta"])
    # the wave height stays within 0.15 of the depth at the wavemaker (or at
    # the 0.5 m floor), the bound that keeps the wavemaker's source region
    # stable in the reference's algorithm
    hs = np.array([p["Hmo"] for p, _, _ in m])
    dep = np.array([p["DEP_WK"] for p, _, _ in m])
    assert (hs <= np.maximum(0.5, 0.15 * dep) + 1e-12).all()
    # the same seed gives the same members
    m2 = fw.cases.ensemble_members(8, seed=1)
    assert all(a[0] == b[0] and np.array_equal(a[1], b[1]) for a, b in zip(m[:8], m2))


def test_max_runup_measure(fw):
    depth = np.array([[2.0, 1.0, -0.5, -1.0, -2.0]]).T.repeat(3, axis=1)  # x = 5 cells, y = 3
    hm = np.zeros((11, 9))
    hm[3:-3, 3:-3] = np.array([[0.3, 0.4, 0.6, 0.9, 1.0]]).T.repeat(3, axis=1)
    # wet land: -0.5 (0.6 > 0.5); not -1.0 (0.9 < 1.0); not -2.0
    assert fw.max_runup(hm, depth) == 0.5
    assert fw.max_runup(np.zeros((11, 9)), depth) == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("precision,single", [("MIXED", False), ("FP64", False), ("MIXED", True), ("FP64", True)])
def test_ensemble_equals_single_runs(fw, precision, single):
    """Members stepped together (round robin on their streams, or as one
    parent graph per two steps) equal the same runs stepped alone."""
    members = fw.cases.ensemble_members(5, seed=7, nfreq=8, ntheta=4, cells_range=(48 * 48, 128 * 96))
    ens = fw.Ensemble(members, precision=precision, single_launch=single, autotune=single)
    st = ens.step(30)
    assert st == [0] * 5
    st = ens.step(11)  # an odd count as well
    assert st == [0] * 5
    runup = ens.max_runup()
    fields = [(s.get("Eta"), s.get("HeightMax"), s.scalar("TIME")) for s in ens.solvers]
    ens.close()
    for k, (p, d, ph) in enumerate(members):
        q = fw.with_defaults(p)
        q["OUT_Hmax"] = True
        s = fw.Solver(q, precision=precision)
        s.init(d, phases=ph)
        s.step(41)
        assert s.scalar("TIME") == fields[k][2]
        assert np.array_equal(s.get("Eta"), fields[k][0])
        assert np.array_equal(s.get("HeightMax"), fields[k][1])
        assert fw.max_runup(s.get("HeightMax"), d) == runup[k]
        s.close()
