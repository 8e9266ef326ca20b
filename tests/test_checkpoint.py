"""Checkpoint / restore (fw_checkpoint, fw_restore): the run-state
counterpart of the reference's HOT_START restart (mod_global.F:387,
io.F:805, main.F:189).  A run restored from a checkpoint into a fresh
context must continue bit for bit as the run that wrote it: fields, masks,
breaking ages, TIME and DT, the statistics with their compensation terms and
the JON_2D wavemaker.  Contexts with other parameters and malformed files
are refused."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ("Eta", "U", "V", "HU", "HV", "Ubar", "Vbar", "H", "MASK", "MASK9", "AGE", "nu_break")
STATS = ("HeightMax", "HeightMin", "VelocityMax", "MomentumFluxMax", "ETAmean", "Umean", "Vmean", "ETA2mean",
         "SigWaveHeight", "WaveHeightAve", "WaveHeightRMS", "Emax", "Emin", "Num_Zero_Up", "ROLLER_FLUX",
         "UNDERTOW_U", "UNDERTOW_V")


def _barred(fw):
    # JON_2D wavemaker (band tables), breaking on a bar, every statistic on
    p, d, ph, _ = fw.cases.barred_beach(480, 64, 1.0, seed=4, wk_from_shore=120.0)
    p.update({"ROLLER": True, "UNDERTOW": True, "STEADY_TIME": 0.0, "T_INTV_mean": 2.0, "OUT_Hmax": True,
              "OUT_Hmin": True, "OUT_Umax": True, "OUT_MFmax": True})
    return p, d, ph


def _snapshot(s):
    out = {n: s.get(n) for n in STATE + STATS}
    out["TIME"] = s.scalar("TIME")
    out["DT"] = s.scalar("DT")
    return out


def _same(a, b):
    assert a["TIME"] == b["TIME"] and a["DT"] == b["DT"]
    for n in STATE + STATS:
        assert np.array_equal(a[n], b[n], equal_nan=True), n


@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
@pytest.mark.parametrize("first", [517, 520])  # odd / even: the MASK and AGE buffers in either orientation
def test_restored_run_continues_bit_for_bit(fw, tmp_path, precision, first):
    p, d, ph = _barred(fw)
    q = fw.with_defaults(p)
    path = str(tmp_path / "run.ckpt")
    a = fw.Solver(q, precision=precision)
    a.init(d, phases=ph)
    assert a.step(first) == 0
    assert (a.get("ROLLER_FLUX") != 0).any()  # breaking has started
    a.checkpoint(path)
    assert a.step(45) == 0
    want = _snapshot(a)
    a.close()
    b = fw.Solver(q, precision=precision)
    b.restore(path)  # no init()
    assert b.step(45) == 0
    _same(_snapshot(b), want)
    b.close()
    # into a context already running another state, stepped one step at a
    # time (no graph) and under another launch tuning
    c = fw.Solver(q, precision=precision)
    c.init(d, phases=ph)
    c.step(3)
    c.restore(path)
    t = c.tuning()
    t["update"] = (128, 1)
    c.set_tuning(t)
    for _ in range(45):
        assert c.step(1) == 0
    _same(_snapshot(c), want)
    c.close()


def test_restore_refuses_other_runs_and_bad_files(fw, tmp_path):
    p, d, _ = fw.cases.planar_beach(Mglob=96, Nglob=40, seed=2)
    q = fw.with_defaults(p)
    path = str(tmp_path / "a.ckpt")
    a = fw.Solver(q, precision="MIXED")
    a.init(d)
    a.step(10)
    a.checkpoint(path)
    want = _snapshot_small(a)
    a.close()
    # other parameters, other precision, other size
    for change, prec in (({"CFL": 0.4}, "MIXED"), ({}, "FP64"), ({"Nglob": 41}, "MIXED")):
        r = dict(q)
        r.update(change)
        s = fw.Solver(fw.with_defaults(r), precision=prec)
        with pytest.raises(fw.FwError) as e:
            s.restore(path)
        assert e.value.status == -3  # FW_ERR_BAD_PARAM
        s.close()
    s = fw.Solver(q, precision="MIXED")
    # missing, foreign and truncated files
    with pytest.raises(fw.FwError) as e:
        s.restore(str(tmp_path / "absent.ckpt"))
    assert e.value.status == -9  # FW_ERR_IO
    junk = tmp_path / "junk.ckpt"
    junk.write_bytes(b"not a checkpoint" * 64)
    with pytest.raises(fw.FwError) as e:
        s.restore(str(junk))
    assert e.value.status == -9
    raw = open(path, "rb").read()
    cut = tmp_path / "cut.ckpt"
    cut.write_bytes(raw[: len(raw) - 1000])
    with pytest.raises(fw.FwError) as e:
        s.restore(str(cut))
    assert e.value.status == -9
    with pytest.raises(fw.FwError) as e:  # the failed read left it un-initialised
        s.step(1)
    assert e.value.status == -7  # FW_ERR_NOT_READY
    long_ = tmp_path / "long.ckpt"
    long_.write_bytes(raw + b"\0")
    with pytest.raises(fw.FwError) as e:
        s.restore(str(long_))
    assert e.value.status == -9
    # and the good file still restores into the same context
    s.restore(path)
    got = _snapshot_small(s)
    for n in want:
        assert np.array_equal(got[n], want[n]), n
    with pytest.raises(fw.FwError) as e:
        s.checkpoint(os.path.join(str(tmp_path), "no_such_dir", "x.ckpt"))
    assert e.value.status == -9
    s.close()


def _snapshot_small(s):
    out = {n: s.get(n) for n in ("Eta", "U", "V", "MASK")}
    out["TIME"] = np.array(s.scalar("TIME"))
    return out
