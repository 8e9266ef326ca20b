"""fw_estimate_dt_device: the CFL time step on device arrays the caller owns,
with no device allocation inside the call.

It exists for callers that cannot call cudaMalloc: a Fortran host whose
device arrays belong to its OpenACC or CUDA Fortran runtime, a code bound to
a fixed memory pool, or a loop in which allocation is forbidden.  Its scratch
is one static device array, so these checks compare it, for two calls in a
row each, with the context entry point fw_estimate_dt on the same U, V, H,
with the oracle's ESTIMATE_DT (also with the DT_fixed halving and without
TIME), and with a numpy minimum on a grid of more than 1024 scratch blocks.
They also check that a grid beyond the stated maximum and host pointers are
refused before any work.  The test allocates its own device arrays with
torch; the entry point does not.  This file is collected last, and passes
alone or after the others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FW_ERR_BAD_PARAM = -3


def _entry(fw):
    L = fw.load_library()
    f = L.fw_estimate_dt_device
    dp, vp = ctypes.c_double, ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, vp, vp, vp, dp, dp, dp, vp, vp, vp]
    f.restype = ctypes.c_int
    return f


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    torch.cuda.set_device(0)
    return torch


def _call(fw, torch, f, Mloc, Nloc, dx, dy, U, V, H, mdf, cfl, dt_fixed, time0, with_time=True):
    """U, V, H: Mloc x Nloc arrays; returns (DT, TIME or None)."""
    dev = torch.device("cuda:0")
    dU, dV, dH = (torch.from_numpy(np.asarray(a, dtype=np.float64).ravel(order="F").copy()).to(dev)
                  for a in (U, V, H))
    out = torch.tensor([-1.0, time0], dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    rc = f(Mloc, Nloc, dx, dy, dU.data_ptr(), dV.data_ptr(), dH.data_ptr(), mdf, cfl, dt_fixed,
           out.data_ptr(), (out.data_ptr() + 8) if with_time else None, stream)
    assert rc == 0, fw.FW_ERRORS.get(rc, rc)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    return float(o[0]), (float(o[1]) if with_time else None)


def test_no_alloc_dt_equals_context_entry_point(fw):
    torch = _torch()
    f = _entry(fw)
    params, depth, _ = fw.cases.planar_beach(Mglob=96, Nglob=64)
    p = fw.with_defaults(params)
    s = fw.Solver(p, precision="FP64")
    s.init(depth)
    for call in range(2):
        s.step(3 + 4 * call)
        time0 = s.scalar("TIME")
        s.estimate_dt()
        dt_ctx, time_ctx = s.scalar("DT"), s.scalar("TIME")
        dt_dev, time_dev = _call(fw, torch, f, s.Mloc, s.Nloc, p["DX"], p["DY"], s.get("U"), s.get("V"),
                                 s.get("H"), p["MinDepthFrc"], p["CFL"], 0.0, time0)
        assert dt_ctx > 0.0
        # the same arithmetic per cell and an exact minimum: bit for bit
        assert dt_dev == dt_ctx, (call, dt_dev, dt_ctx)
        assert time_dev == time_ctx, (call, time_dev, time_ctx)
    s.close()


@pytest.mark.parametrize("dt_fixed,with_time", [(0.0, False), (0.37, True), (0.37, False)])
def test_no_alloc_dt_equals_oracle(fw, oracle_mod, dt_fixed, with_time):
    """The oracle's ESTIMATE_DT (misc.F:216-296) on the same arrays, with and
    without the DT_fixed halving and TIME, two calls in a row."""
    torch = _torch()
    f = _entry(fw)
    fo = oracle_mod
    params, _, _ = fw.cases.planar_beach(Mglob=60, Nglob=40)
    p = fw.with_defaults(params)
    if dt_fixed > 0.0:
        p["DT_fixed"] = dt_fixed
    o = fo.Oracle(p)
    rng = np.random.default_rng(11)
    for call in range(2):
        U = rng.normal(0.0, 0.8, size=(o.Mloc, o.Nloc))
        V = rng.normal(0.0, 0.8, size=(o.Mloc, o.Nloc))
        H = rng.uniform(-0.5, 6.0, size=(o.Mloc, o.Nloc))
        o["U"][:] = U
        o["V"][:] = V
        o["H"][:] = H
        time0 = 12.5 + call
        o.set_scalar("TIME", time0)
        o.call("estimate_dt")
        dt_ref, time_ref = o.scalar("DT"), o.scalar("TIME")
        dt_dev, time_dev = _call(fw, torch, f, o.Mloc, o.Nloc, p["DX"], p["DY"], U, V, H, p["MinDepthFrc"],
                                 p["CFL"], dt_fixed, time0, with_time)
        assert dt_ref > 0.0
        assert dt_dev == dt_ref, (call, dt_dev, dt_ref)
        if with_time:
            assert time_dev == time_ref, (call, time_dev, time_ref)
    o.close()


def test_no_alloc_dt_many_blocks(fw):
    """2048 x 1100 cells: 1100 scratch blocks, so the final reduction's
    strided loop over more than 1024 block minima runs; checked against a
    numpy minimum of the CFL formula, two calls in a row."""
    torch = _torch()
    f = _entry(fw)
    M, N, dx, dy, mdf, cfl = 2048, 1100, 1.5, 2.0, 0.1, 0.5
    rng = np.random.default_rng(5)
    for call in range(2):
        U = rng.normal(0.0, 1.0, size=(M, N))
        V = rng.normal(0.0, 1.0, size=(M, N))
        H = rng.uniform(0.0, 8.0, size=(M, N))
        # the fastest cell sits in a block beyond the first 1024
        U[M - 5 - call, N - 3] = 40.0 + call
        c = np.sqrt(9.81 * np.maximum(H, mdf))
        tmp3 = min((dx / (np.abs(U) + c)).min(), (dy / (np.abs(V) + c)).min())
        dt_dev, time_dev = _call(fw, torch, f, M, N, dx, dy, U, V, H, mdf, cfl, 0.0, 1.0)
        assert dt_dev == cfl * tmp3, (call, dt_dev, cfl * tmp3)
        assert time_dev == 1.0 + dt_dev


def test_no_alloc_dt_refuses_bad_arguments(fw):
    torch = _torch()
    f = _entry(fw)
    # 16384 x 8193 cells is one cell-block past the maximum; the call returns
    # FW_ERR_BAD_PARAM before it touches any pointer or launches anything
    dummy = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    ptr = dummy.data_ptr()
    rc = f(16384, 8193, 1.0, 1.0, ptr, ptr, ptr, 0.1, 0.5, 0.0, ptr, ptr, None)
    assert rc == FW_ERR_BAD_PARAM
    # host arrays in place of device arrays are refused before any launch
    host = np.zeros(64, dtype=np.float64)
    hp = host.ctypes.data
    dev = torch.zeros(64, dtype=torch.float64, device="cuda:0")
    dptr = dev.data_ptr()
    assert f(8, 8, 1.0, 1.0, hp, dptr, dptr, 0.1, 0.5, 0.0, dptr, None, None) == FW_ERR_BAD_PARAM
    assert f(8, 8, 1.0, 1.0, dptr, dptr, dptr, 0.1, 0.5, 0.0, hp, None, None) == FW_ERR_BAD_PARAM
    assert f(8, 8, 1.0, 1.0, dptr, dptr, dptr, 0.1, 0.5, 0.0, dptr, hp, None) == FW_ERR_BAD_PARAM
    # the library still works after the refusals
    dt, _ = _call(fw, torch, f, 8, 8, 1.0, 1.0, np.zeros((8, 8)), np.zeros((8, 8)), np.ones((8, 8)),
                  0.1, 0.5, 0.0, 0.0, with_time=False)
    assert dt == 0.5 * (1.0 / np.sqrt(9.81))
