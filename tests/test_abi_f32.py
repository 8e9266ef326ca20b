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


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_f32_multi_field_transfers(fw, precision):
    """fw_set_fields_f32 / fw_get_fields_f32 move several fields at once and
    equal the one-field calls; "Depth" among them keeps the mixed build's
    double copy of the total-depth tests in step (the run goes on equally).
    Pageable host arrays take the copy path; page-locked ones are read and
    written in place by the transfer kernels (mixed build): both equal."""
    import ctypes
    torch = pytest.importorskip("torch")
    params, depth, _ = fw.cases.planar_beach(Mglob=70, Nglob=44, seed=6)
    p = fw.with_defaults(params)
    eta, u, v = fw.cases.random_state(70, 44, seed=7)

    def host_array(shape, pinned):
        if not pinned:
            return np.zeros(shape, dtype=np.float32, order="F")
        # a Fortran-ordered view of page-locked memory
        return torch.zeros((shape[1], shape[0]), dtype=torch.float32, pin_memory=True).numpy().T

    runs = []
    for mode in ("single", "pageable", "pinned"):
        multi, pinned = mode != "single", mode == "pinned"
        s = fw.Solver(p, precision=precision)
        s.init(depth, eta, u, v)
        s.step(2)
        names = ("Eta", "U", "Vbar", "Depth")
        arrs = {}
        for n in names:
            arrs[n] = host_array(s.shape(n), pinned)
            arrs[n][...] = s.get_f32(n) * np.float32(1.0 + 1e-3)
        if multi:
            cn = (ctypes.c_char_p * 4)(*[n.encode() for n in names])
            hp = (ctypes.c_void_p * 4)(*[arrs[n].ctypes.data for n in names])
            assert s.L.fw_set_fields_f32(s.ctx, 4, cn, hp) == 0
            outs = {n: host_array(s.shape(n), pinned) for n in names}
            op = (ctypes.c_void_p * 4)(*[outs[n].ctypes.data for n in names])
            assert s.L.fw_get_fields_f32(s.ctx, 4, cn, op) == 0
            for n in names:
                assert np.array_equal(outs[n], s.get_f32(n)), n
                assert np.array_equal(outs[n], arrs[n]), n
        else:
            for n in names:
                s.set_f32(n, arrs[n])
        assert s.step(3, check=False) == 0
        runs.append(s.get("Eta"))
        s.close()
    assert np.array_equal(runs[0], runs[1])
    assert np.array_equal(runs[0], runs[2])
