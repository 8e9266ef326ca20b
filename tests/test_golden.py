"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py
from the oracle): whole steps of three small cases — WK_REG on a periodic
planar beach from a random state, JON_2D over the elliptic shoal with walls,
and a breaking case from a steep random state.

CPU: the oracle still reproduces every fixture bit for bit (a change of the
restatement shows up here).  GPU: the FP64 kernels agree with the fixtures
to 1e-9 of each field's scale after the same steps, MASK and MASK9 exactly.
"""
import ast
import glob
import os

import numpy as np
import pytest

from helpers import G

HERE = os.path.dirname(os.path.abspath(__file__))
# the oracle's fixtures (berkhoff.npz holds reference data, tests/test_berkhoff.py)
FIXTURES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                  if not os.path.basename(p).startswith("berkhoff"))
FIELDS = ("Eta", "U", "V", "Ubar", "Vbar", "HU", "HV", "H", "MASK", "MASK9", "AGE", "nu_break",
          "P", "Q", "Depthx", "Depthy", "HeightMax")


def _load(path):
    z = np.load(path)
    params = dict(ast.literal_eval(str(z["params"])))
    inputs = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    outputs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return params, inputs, outputs, int(z["nsteps"])


def test_fixtures_present():
    assert len(FIXTURES) == 3


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_reproduces_fixture(oracle_mod, fw, path):
    params, inp, out, n = _load(path)
    o = oracle_mod.Oracle(fw.with_defaults(params))
    o["Depth"][G:-G, G:-G] = inp["depth"]
    if "eta" in inp:
        o["Eta"][G:-G, G:-G] = inp["eta"]
        o["U"][G:-G, G:-G] = inp["u"]
        o["V"][G:-G, G:-G] = inp["v"]
    if "phases" in inp:
        o.set_phases(np.asfortranarray(inp["phases"]))
    o.init()
    for _ in range(n):
        assert o.step() == 0
    for name in FIELDS:
        assert np.array_equal(np.asarray(o[name]), out[name]), name
    assert o.scalar("TIME") == float(out["TIME"])
    o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_gpu_fp64_matches_fixture(fw, path):
    params, inp, out, n = _load(path)
    p = fw.with_defaults(params)
    p["OUT_Hmax"] = True
    s = fw.Solver(p, precision="FP64")
    s.init(inp["depth"], inp.get("eta"), inp.get("u"), inp.get("v"),
           np.asfortranarray(inp["phases"]) if "phases" in inp else None)
    assert s.step(n) == 0
    for name in FIELDS:
        a, b = s.get(name), out[name]
        if name in ("MASK", "MASK9"):
            assert np.array_equal(a, b), name
            continue
        scale = max(float(np.abs(b).max()), 1e-6)
        e = float(np.abs(a - b).max()) / scale
        assert e <= 1e-9, "%s: %.3e" % (name, e)
    assert abs(s.scalar("TIME") - float(out["TIME"])) <= 1e-12 * float(out["TIME"])
    s.close()
