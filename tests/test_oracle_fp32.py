"""The oracle's single-precision build, which bench.py times as the CPU
baseline and as the reference arm (the reference's default build is single
precision, REAL(SP) = REAL(4), mod_param.F:58-68): it computes the same run
as the FP64 restatement to float rounding.  A breaking beach with a
wavemaker, dispersion and wet/dry steps in both builds from the same start;
the float build's arrays are float32, its time steps and its eta stay within
float rounding of the double build's."""
import numpy as np

from helpers import G, sloped_beach


def _run(fw, oracle_mod, fp32, nsteps):
    p, _, _ = fw.cases.planar_beach(Mglob=64, Nglob=24, seed=5)
    p.update({"PERIODIC": False, "Cbrk1": 0.2, "Cbrk2": 0.1})
    p = fw.with_defaults(p)
    depth = sloped_beach(64, 24, h0=3.0, h1=-0.8, seed=6)
    eta, u, v = fw.cases.random_state(64, 24, seed=7, eta_amp=0.1, u_amp=0.2)
    o = oracle_mod.Oracle(p, threads=2, fp32=fp32)
    o["Depth"][G:-G, G:-G] = depth
    o["Eta"][G:-G, G:-G] = eta
    o["U"][G:-G, G:-G] = u
    o["V"][G:-G, G:-G] = v
    o.init()
    dts = []
    for _ in range(nsteps):
        o.step()
        dts.append(o.scalar("DT"))
    out = {"Eta": np.array(o["Eta"][G:-G, G:-G], dtype=np.float64), "MASK": np.array(o["MASK"][G:-G, G:-G]),
           "real": o.real, "DT": np.array(dts), "TIME": o.scalar("TIME")}
    o.close()
    return out


def test_single_precision_build_follows_the_double_one(fw, oracle_mod):
    a = _run(fw, oracle_mod, True, 40)
    b = _run(fw, oracle_mod, False, 40)
    assert a["real"] == np.float32 and b["real"] == np.float64
    assert np.allclose(a["DT"], b["DT"], rtol=1e-6, atol=0.0)
    assert abs(a["TIME"] - b["TIME"]) <= 1e-6 * b["TIME"]
    wet = (a["MASK"] > 0) & (b["MASK"] > 0)
    d = a["Eta"][wet] - b["Eta"][wet]
    assert np.isfinite(a["Eta"]).all()
    # float rounding: about 3e-8 m RMS against 0.05 m of eta after 40 steps
    assert float(np.sqrt(np.mean(d * d))) <= 1e-6
    assert float(np.sum(a["MASK"] != b["MASK"])) <= 0.01 * a["MASK"].size
