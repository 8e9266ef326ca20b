"""Captured steps (fw_step): pairs of steps replay one two-step graph, single
steps one of two one-step graphs (one per orientation of the MASK and AGE
ping-pong buffers, which a step flips).  Any split of a run into calls must
compute the same values bit for bit as one call, also when the tuning or a
scalar changes between calls (which re-captures)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("Eta", "U", "V", "HU", "HV", "Ubar", "Vbar", "MASK", "MASK9", "AGE", "nu_break", "ROLLER_FLUX")


def _case(fw):
    p, d, ph, _ = fw.cases.barred_beach(480, 64, 1.0, seed=4, wk_from_shore=120.0)
    p.update({"ROLLER": True, "STEADY_TIME": 0.0, "T_INTV_mean": 4.0})
    return fw.with_defaults(p), d, ph


def _state(s):
    out = {n: s.get(n) for n in FIELDS}
    out["TIME"] = s.scalar("TIME")
    return out


@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
def test_any_split_of_a_run_is_the_same(fw, precision):
    q, d, ph = _case(fw)
    a = fw.Solver(q, precision=precision)
    a.init(d, phases=ph)
    assert a.step(560) == 0
    want = _state(a)
    a.close()
    assert (want["ROLLER_FLUX"] != 0).any()
    b = fw.Solver(q, precision=precision)
    b.init(d, phases=ph)
    done, k = 0, 0
    pattern = (1, 1, 1, 2, 1, 3, 1, 1, 2, 2, 1, 5)
    t = b.tuning()
    while done < 560:
        n = min(pattern[k % len(pattern)], 560 - done)
        assert b.step(n) == 0
        done += n
        k += 1
        if k == 40:  # re-capture under another tuning
            t["update"] = (128, 1)
            b.set_tuning(t)
        if k == 80:
            b.set_scalar("EtaBlowVal", 1e6)
    got = _state(b)
    assert got["TIME"] == want["TIME"]
    for n in FIELDS:
        assert np.array_equal(got[n], want[n]), n
    b.close()
