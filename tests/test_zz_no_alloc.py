"""fw_estimate_dt_device: the CFL time step on device arrays the caller owns,
with no device allocation inside the call.

It exists for callers that cannot call cudaMalloc: a Fortran host whose
device arrays belong to its OpenACC or CUDA Fortran runtime, a code bound to
a fixed memory pool, or a loop in which allocation is forbidden.  Its scratch
is one static device array, so these checks compare it with the context
entry point fw_estimate_dt on the same U, V, H, for two calls in a row, and
check that a grid beyond its stated maximum is refused before any work.
The test allocates its own device arrays with torch; the entry point does
not.  This file is collected last, and passes alone or after the others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-11  # the relative tolerance of the FP64 parity tests


def _entry(fw):
    L = fw.load_library()
    f = L.fw_estimate_dt_device
    dp, vp = ctypes.c_double, ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, vp, vp, vp, dp, dp, dp, vp, vp, vp]
    f.restype = ctypes.c_int
    return f


def _device_dt(fw, torch, f, s, p, time0):
    dev = torch.device("cuda:0")
    U, V, H = (torch.from_numpy(np.asfortranarray(s.get(n)).ravel(order="F").copy()).to(dev)
               for n in ("U", "V", "H"))
    out = torch.tensor([0.0, time0], dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    rc = f(s.Mloc, s.Nloc, p["DX"], p["DY"], U.data_ptr(), V.data_ptr(), H.data_ptr(),
           p["MinDepthFrc"], p["CFL"], 0.0, out.data_ptr(), out.data_ptr() + 8, stream)
    assert rc == 0, fw.FW_ERRORS.get(rc, rc)
    torch.cuda.synchronize()
    return float(out[0]), float(out[1])


def test_no_alloc_dt_matches_context_entry_point(fw):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    torch.cuda.set_device(0)
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
        dt_dev, time_dev = _device_dt(fw, torch, f, s, p, time0)
        assert dt_ctx > 0.0
        assert abs(dt_dev - dt_ctx) <= TOL * dt_ctx, (call, dt_dev, dt_ctx)
        assert abs(time_dev - time_ctx) <= TOL * time_ctx, (call, time_dev, time_ctx)
    s.close()


def test_no_alloc_dt_rejects_grid_beyond_maximum(fw):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    f = _entry(fw)
    # 16384 x 8193 cells is one cell-block past the maximum; the call returns
    # FW_ERR_BAD_PARAM before it touches any pointer or launches anything
    dummy = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    ptr = dummy.data_ptr()
    rc = f(16384, 8193, 1.0, 1.0, ptr, ptr, ptr, 0.1, 0.5, 0.0, ptr, ptr, None)
    assert rc == -3
