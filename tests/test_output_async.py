"""Asynchronous output (fw_output_begin / fw_output_wait / fw_output_done):
PREVIEW's field transfers (io.F:4304-4621) staged while later steps run.
The snapshot holds the state after the steps enqueued before the call, in
fw_get_field's layout and types, whatever runs after it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ("Eta", "U", "V", "MASK", "P", "Gy", "HeightMax", "ETAmean")


@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
def test_snapshot_is_the_state_at_the_call(fw, precision):
    p, d, _ = fw.cases.planar_beach(Mglob=120, Nglob=56, seed=6)
    p.update({"OUT_Hmax": True, "STEADY_TIME": 0.0, "T_INTV_mean": 1.0})
    s = fw.Solver(fw.with_defaults(p), precision=precision)
    s.init(d)
    s.step(30)
    want = {n: s.get(n) for n in NAMES}
    out = s.output_begin(NAMES)
    s.step_async(40)  # runs while the copies proceed
    got = out.wait()
    assert s.step_wait() == 0
    for n in NAMES:
        assert got[n].dtype == want[n].dtype and got[n].shape == want[n].shape, n
        assert np.array_equal(got[n], want[n]), n
    assert not np.array_equal(s.get("Eta"), want["Eta"])  # the run went on
    # back to back: the second call waits for the first one's copies
    a = s.output_begin(("Eta",))
    b = s.output_begin(("Eta", "U"))
    assert a.done()
    now = s.get("Eta")
    assert np.array_equal(a.wait()["Eta"], now) and np.array_equal(b.wait()["Eta"], now)
    assert b.done()
    s.close()


def test_unknown_or_switched_off_fields_are_refused(fw):
    p, d, _ = fw.cases.planar_beach(Mglob=64, Nglob=32, seed=1)
    s = fw.Solver(fw.with_defaults(p), precision="MIXED")
    s.init(d)
    for bad in (("Eta", "nope"), ("HeightMin",)):  # HeightMin is off in this run
        with pytest.raises(fw.FwError) as e:
            s.output_begin(bad)
        assert e.value.status == -3
    assert s.output_begin(("Eta",)).wait()["Eta"].shape == (70, 38)
    s.close()


@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
def test_batched_transfers_equal_single_ones(fw, precision):
    """fw_set_fields / fw_get_fields move the same values as fw_set_field /
    fw_get_field, masks included."""
    p, d, _ = fw.cases.planar_beach(Mglob=90, Nglob=40, seed=3)
    s = fw.Solver(fw.with_defaults(p), precision=precision)
    s.init(d)
    s.step(12)
    names = ("Eta", "U", "V", "Ubar", "Vbar", "MASK", "P")
    before = s.get_fields(names)
    for n in names:
        assert np.array_equal(before[n], s.get(n)), n
    rng = np.random.default_rng(1)
    new = {n: before[n] + (0 if n == "MASK" else 1e-3 * rng.standard_normal(before[n].shape)) for n in names}
    new["MASK"] = before["MASK"].copy()
    new["MASK"][5, 7] = 1 - new["MASK"][5, 7]
    s.set_fields(new)
    ref = fw.Solver(fw.with_defaults(p), precision=precision)
    ref.init(d)
    ref.step(12)
    for n in names:
        ref.set(n, new[n])
    for n in names:
        assert np.array_equal(s.get(n), ref.get(n)), n
    assert s.step(3) == 0 and ref.step(3) == 0
    for n in ("Eta", "U", "MASK"):
        assert np.array_equal(s.get(n), ref.get(n)), n
    with pytest.raises(fw.FwError):
        s.set_fields({"Eta": new["Eta"], "nope": new["U"]})
    s.close()
    ref.close()
