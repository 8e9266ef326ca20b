"""The barred-beach configuration (1:40 slope, Gaussian bar cut by rip
channels, normal-incidence JONSWAP, wetting-drying and breaking) at a small
size: the generator's geometry (CPU) and mixed precision against FP64 on the
GPU once the waves have reached the bar and the shoreline."""
import numpy as np
import pytest

from helpers import G


def test_geometry(fw):
    p, d, ph, rips = fw.cases.barred_beach(600, 400, 1.0, seed=3)
    x_shore = 600 - 300.0
    assert len(rips) == 4 and all(0.05 * 400 <= c <= 0.95 * 400 for c in rips)
    assert all(abs(a - b) >= 40.0 for i, a in enumerate(rips) for b in rips[i + 1:])
    i_bar = int(x_shore - 80.0)
    j_rip = int(rips[0])
    j_bar = [j for j in range(400) if all(abs(j + 0.5 - c) > 25.0 for c in rips)][0]
    # the bar rises 1.5 m above the plain slope between channels, not in one
    plain = (x_shore - (i_bar + 0.5)) / 40.0
    assert abs((plain - d[i_bar, j_bar]) - 1.5) < 0.05
    assert abs(d[i_bar, j_rip] - plain) < 1e-9
    assert (d[-1, :] < 0).all() and d.max() <= 12.0


@pytest.mark.gpu
def test_mixed_vs_fp64_barred_beach(fw):
    p, d, ph, _ = fw.cases.barred_beach(480, 256, 1.0, seed=4, wk_from_shore=120.0)
    p = fw.with_defaults(p)
    p["OUT_Hmax"] = True
    res = {}
    for prec in ("FP64", "MIXED"):
        s = fw.Solver(p, precision=prec)
        s.init(d, phases=ph)
        s.step(500)
        res[prec] = {k: s.get(k)[G:-G, G:-G] for k in ("Eta", "MASK", "HeightMax", "AGE")}
        res[prec]["TIME"] = s.scalar("TIME")
        s.close()
    a, b = res["MIXED"], res["FP64"]
    assert abs(a["TIME"] - b["TIME"]) <= 1e-3 * b["TIME"]
    wet = (a["MASK"] > 0) & (b["MASK"] > 0)
    assert (b["AGE"] > 0).any()  # waves break on the bar or the beach
    rms = float(np.sqrt(np.mean((a["Eta"] - b["Eta"])[wet] ** 2)))
    assert rms <= 1e-4, rms
    assert float(np.sum(a["MASK"] != b["MASK"])) <= 0.002 * a["MASK"].size
    ra = fw.max_runup(np.pad(a["HeightMax"], G), d)
    rb = fw.max_runup(np.pad(b["HeightMax"], G), d)
    assert rb > 0.0 and abs(ra - rb) <= 0.05 * rb + 0.01
