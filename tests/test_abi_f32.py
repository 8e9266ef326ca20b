"""fw_get_field_f32 / fw_set_field_f32: the float host arrays of a
single-precision host build (REAL(SP) = 4-byte reals, mod_param.F:58-68).

Out of the FP64 build a field arrives rounded to nearest float, exactly as
numpy rounds the double transfer; out of the mixed build it is the stored
float itself.  In both builds a float array written with fw_set_field_f32
reads back unchanged.  Masks keep their int32 transfers and are refused.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_f32_transfers(fw, precision):
    params, depth, _ = fw.cases.planar_beach(Mglob=70, Nglob=44, seed=6)
    s = fw.Solver(fw.with_defaults(params), precision=precision)
    eta, u, v = fw.cases.random_state(70, 44, seed=7)
    s.init(depth, eta, u, v)
    s.step(3)
    for name in ("Eta", "U", "V", "Ubar", "H", "P", "Gy", "Depthx", "AGE"):
        d = s.get(name)
        f = s.get_f32(name)
        assert f.dtype == np.float32 and f.shape == d.shape
        assert np.array_equal(f, d.astype(np.float32)), name
    rng = np.random.default_rng(9)
    keep = {n: s.get(n) for n in ("Eta", "Vbar", "Q")}
    for name in ("Eta", "Vbar", "Q"):
        a = rng.normal(size=s.shape(name)).astype(np.float32)
        s.set_f32(name, a)
        assert np.array_equal(s.get(name), a.astype(np.float64)), name
        assert np.array_equal(s.get_f32(name), a), name
    with pytest.raises(fw.FwError) as e:
        s.get_f32("MASK")
    assert e.value.status == -3
    # the run goes on from its own state written back as floats
    for name, a in keep.items():
        s.set_f32(name, a.astype(np.float32))
    assert s.step(2, check=False) == 0
    s.close()
