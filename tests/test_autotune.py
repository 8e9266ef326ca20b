"""Launch-shape autotuning (fw_autotune, fw_set_tuning): no reference
counterpart.  Every candidate shape must compute the same values bit for bit
(the tuned kernels are per-cell or per-face), the tuning must leave a run's
state as it found it, and shapes outside the compiled candidates are
refused."""
import numpy as np
import pytest

FIELDS = ("Eta", "U", "V", "HU", "HV", "Ubar", "Vbar", "MASK", "MASK9", "AGE")


def _run(fw, precision, nsteps, tuning=None, autotune_after=None):
    # 200 x 72 cells: no tile or block shape divides the grid evenly
    p, d, _ = fw.cases.planar_beach(Mglob=200, Nglob=72, seed=4)
    s = fw.Solver(fw.with_defaults(p), precision=precision)
    s.init(d)
    if tuning is not None:
        s.set_tuning(tuning)
    if autotune_after is None:
        s.step(nsteps)
    else:
        s.step(autotune_after)
        before = {n: s.get(n) for n in FIELDS}
        t_before = s.scalar("TIME")
        s.autotune(fresh=True)
        for n in FIELDS:
            assert np.array_equal(s.get(n), before[n]), n
        assert s.scalar("TIME") == t_before
        s.step(nsteps - autotune_after)
    out = {n: s.get(n) for n in FIELDS}
    out["TIME"] = s.scalar("TIME")
    out["tuning"] = s.tuning()
    s.close()
    return out


def _same(a, b):
    assert a["TIME"] == b["TIME"]
    for n in FIELDS:
        assert np.array_equal(a[n], b[n]), n


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
def test_every_launch_shape_computes_the_same(fw, precision):
    ref = _run(fw, precision, 24)
    alts = [
        {"disp_a": (64, 4), "disp_b": (128, 2), "update": (256, 1), "post_mask_break": (32, 4),
         "maskmul": (64, 2), "flux_x": 16, "flux_y": 16 if precision == "MIXED" else 8},
        {"disp_a": (256, 1), "disp_b": (32, 2), "update": (128, 1), "post_mask_break": (128, 2),
         "maskmul": (32, 8), "flux_x": 32 if precision == "MIXED" else 8, "flux_y": 8 if precision == "MIXED" else 16},
        # the flux tiles staged by TMA
        {"disp_a": (32, 8), "disp_b": (32, 8), "update": (32, 8), "post_mask_break": (32, 8), "maskmul": (32, 8),
         "flux_x": 16, "flux_y": 16, "flux_x_tma": 1, "flux_y_tma": 1},
        {"disp_a": (32, 8), "disp_b": (32, 8), "update": (32, 8), "post_mask_break": (32, 8), "maskmul": (32, 8),
         "flux_x": 8, "flux_y": 32 if precision == "MIXED" else 8, "flux_x_tma": 1, "flux_y_tma": 1},
    ]
    for t in alts:
        out = _run(fw, precision, 24, tuning=t)
        assert out["tuning"] == dict({"flux_x_tma": 0, "flux_y_tma": 0}, **t)
        _same(out, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
def test_autotune_leaves_the_run_unchanged(fw, precision):
    ref = _run(fw, precision, 20)
    tuned = _run(fw, precision, 20, autotune_after=7)
    _same(tuned, ref)
    t = tuned["tuning"]
    for k in ("disp_a", "disp_b", "update", "post_mask_break", "maskmul"):
        bx, by = t[k]
        assert bx % 32 == 0 and bx * by <= 256
    for k in ("flux_x", "flux_y"):
        assert t[k] in ((8, 16, 32) if precision == "MIXED" else (8, 16))
        assert t[k + "_tma"] in (0, 1)


@pytest.mark.gpu
def test_set_tuning_refuses_shapes_that_are_not_built(fw):
    p, d, _ = fw.cases.planar_beach(Mglob=64, Nglob=32)
    s = fw.Solver(fw.with_defaults(p), precision="MIXED")
    s.init(d)
    good = s.tuning()
    for bad in ({"update": (48, 4)}, {"maskmul": (64, 8)}, {"flux_x": 64}, {"flux_y": 12}, {"flux_x_tma": 2}):
        t = dict(good)
        t.update(bad)
        with pytest.raises(fw.FwError):
            s.set_tuning(t)
    assert s.tuning() == good
    s.close()
