"""Generate the golden fixtures of this directory from the oracle (the FP64
C restatement of the reference's hot path).

The reference (Fortran) cannot be compiled on the machines of this project
and ships no test vectors, so these fixtures pin the restatement itself:
the CPU tests check that the oracle still reproduces them bit for bit, the
GPU tests check the FP64 kernels against them.  Each fixture holds its
inputs (interior depth, initial state, JON_2D phases) and the fields after
a few whole steps.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

FIELDS = ("Eta", "U", "V", "Ubar", "Vbar", "HU", "HV", "H", "MASK", "MASK9", "AGE", "nu_break",
          "P", "Q", "Depthx", "Depthy", "HeightMax")
G = 3


def cases(fw):
    """name -> (params, depth, eta, u, v, phases, nsteps)"""
    out = {}
    p, d, _ = fw.cases.planar_beach(Mglob=40, Nglob=24, seed=11)
    st = fw.cases.random_state(40, 24, seed=12, eta_amp=0.08, u_amp=0.15)
    out["planar_wkreg_periodic"] = (p, d, *st, None, 6)
    p, d, ph = fw.cases.shoal_jonswap(Mglob=48, Nglob=32, dx=48.0, seed=13, Nfreq=6, Ntheta=5)
    out["shoal_jonswap_walls"] = (p, d, None, None, None, ph, 12)
    p, d, _ = fw.cases.planar_beach(Mglob=36, Nglob=20, seed=14, PERIODIC=False)
    st = fw.cases.random_state(36, 20, seed=15, eta_amp=0.5, u_amp=0.6, smooth=2.0)
    out["planar_breaking_walls"] = (p, d, *st, None, 8)
    return out


def run_oracle(oracle_mod, fw, params, depth, eta, u, v, phases, nsteps):
    p = fw.with_defaults(params)
    o = oracle_mod.Oracle(p)
    o["Depth"][G:-G, G:-G] = depth
    if eta is not None:
        o["Eta"][G:-G, G:-G] = eta
        o["U"][G:-G, G:-G] = u
        o["V"][G:-G, G:-G] = v
    if phases is not None:
        o.set_phases(phases)
    o.init()
    for _ in range(nsteps):
        assert o.step() == 0
    res = {n: np.array(o[n]) for n in FIELDS}
    res["TIME"] = np.array(o.scalar("TIME"))
    res["DT"] = np.array(o.scalar("DT"))
    o.close()
    return res


def main():
    import __graft_entry__
    import fw_oracle
    fw = __graft_entry__.load_package()
    fw_oracle.build()
    for name, (p, d, eta, u, v, ph, n) in cases(fw).items():
        res = run_oracle(fw_oracle, fw, p, d, eta, u, v, ph, n)
        blob = {"out_" + k: val for k, val in res.items()}
        blob["in_depth"] = d
        blob["nsteps"] = np.array(n)
        if eta is not None:
            blob["in_eta"], blob["in_u"], blob["in_v"] = eta, u, v
        if ph is not None:
            blob["in_phases"] = ph
        blob["params"] = np.array(repr(sorted(p.items())))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **blob)
        print(name, "TIME %.6f" % res["TIME"], "max|eta| %.4f" % np.abs(res["Eta"]).max(),
              "breaking cells", int((res["AGE"] > 0).sum()))


if __name__ == "__main__":
    main()
