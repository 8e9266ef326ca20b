"""The C-ABI library builds, loads without a GPU and exports every function
that include/funwave_gpu.h declares; the parameter block matches the header.
No compute call is made here."""
import ctypes

import pytest


def test_library_exports_every_declared_symbol(fw):
    L = fw.load_library()
    declared = fw.declared_symbols()
    assert len(declared) >= 25
    missing = [n for n in declared if not hasattr(L, n)]
    assert not missing, missing


def test_params_default_matches_reference_defaults(fw):
    L = fw.load_library()
    from funwave_tvd_gb300.solver import FwParams
    p = FwParams()
    L.fw_params_default(ctypes.byref(p))
    assert p.dispersion == 1 and p.viscosity_breaking == 1 and p.show_breaking == 1
    assert p.gamma1 == 1.0 and p.gamma2 == 1.0 and p.gamma3 == 1.0
    assert p.beta_ref == -0.531
    assert (p.cbrk1, p.cbrk2, p.wavemaker_cbrk) == (0.65, 0.35, 1.0)
    assert p.swe_eta_dep == 0.8 and p.cfl == 0.5 and p.froude_cap == 3.0
    assert p.min_depth == 0.1 and p.min_depth_frc == 0.1
    assert p.r_sponge == 0.85 and p.a_sponge == 5.0 and p.delta_wk == 0.5
    assert p.precision == 0


def test_struct_size_matches_header(fw):
    """sizeof(fw_params) from a tiny C program equals the ctypes layout."""
    import os
    import subprocess
    import tempfile
    from funwave_tvd_gb300.solver import FwParams
    inc = os.path.join(os.path.dirname(fw.__file__), "..", "include")
    src = '#include "funwave_gpu.h"\n#include <stdio.h>\nint main(void){printf("%zu", sizeof(fw_params));return 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I", inc, c, "-o", exe], check=True)
        size = int(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert size == ctypes.sizeof(FwParams)


def test_create_fails_cleanly_without_gpu(fw):
    """Without a GPU, fw_create reports FW_ERR_NO_DEVICE (no fallback)."""
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    p, depth, _ = fw.cases.planar_beach(Mglob=16, Nglob=16)
    with pytest.raises(fw.FwError) as e:
        fw.Solver(p)
    assert e.value.status == -8


def test_strerror(fw):
    L = fw.load_library()
    assert L.fw_strerror(-4).decode().startswith("blow-up")
    assert L.fw_strerror(0).decode() == "ok"
    assert L.fw_strerror(-9).decode().startswith("checkpoint file")


def test_output_switches_under_their_input_keys(fw):
    """input.txt names the output switches Hmax, Umean, Radiation, ...
    (io.F:3392-3424); read_input_txt maps them to the OUT_* names, and the
    radiation sums are switched on for Radiation, Umean or Vmean."""
    from funwave_tvd_gb300.solver import params_struct
    deck = "Mglob = 8\nNglob = 8\nDX = 1.0\nDY = 1.0\nHmax = T\nMFmax = T\nUmean = T\nRadiation = F\n"
    p = fw.read_input_txt(deck)
    assert p["OUT_Hmax"] is True and p["OUT_MFmax"] is True and p["OUT_Umean"] is True
    assert p["OUT_Radiation"] is False and "Hmax" not in p
    s = params_struct(p)
    assert s.track_hmax == 1 and s.track_mfmax == 1 and s.track_hmin == 0 and s.track_radiation == 1
    assert params_struct(fw.read_input_txt("Mglob = 8\nNglob = 8\nDX = 1.0\nDY = 1.0\n")).track_radiation == 0


def test_create_refuses_planes_beyond_32_bit_offsets(fw):
    """A grid whose padded plane would hold 2^31 elements or more is refused
    (FW_ERR_UNSUPPORTED) before any device is touched."""
    L = fw.load_library()
    from funwave_tvd_gb300.solver import FwParams
    p = FwParams()
    L.fw_params_default(ctypes.byref(p))
    p.Mglob, p.Nglob, p.DX, p.DY = 2_000_000, 1100, 1.0, 1.0
    h = ctypes.c_void_p()
    assert L.fw_create(ctypes.byref(p), ctypes.byref(h)) == -6
    assert not h.value
