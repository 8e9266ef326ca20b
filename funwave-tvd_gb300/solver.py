"""ctypes binding of ``libfunwave_gpu.so`` (include/funwave_gpu.h).

:class:`Solver` mirrors the reference's driver interface for the hot path:
the unit calls keep the Fortran subroutine names (``cal_dispersion``,
``fluxes``, ``source_terms``, ``estimate_huv``, ``update_mask``,
``wave_breaking``, ``exchange``, ``sponge_damping``, ``estimate_dt``) and
fields are read and written by their MODULE GLOBAL names as Fortran-ordered
numpy arrays with ghost cells.  Errors raise :class:`FwError` carrying the
library status, where the reference would STOP.
"""
import ctypes
import os
import re
import subprocess

import numpy as np

from .params import with_defaults

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
_CSRC = os.path.join(_HERE, "csrc")
_BUILD = os.path.join(_HERE, "_build")
_HEADER = os.path.join(_ROOT, "include", "funwave_gpu.h")
# translation units and their extra flags: the FP64 kernels and the host
# initialisation keep every multiply and add separately rounded (the
# reference's operation order); the mixed-precision kernels may contract and
# use the fast single-precision division and square root (the double
# arithmetic of their line solver is not affected)
_SOURCES = {
    "fw_kernels_f64.cu": ["-fmad=false"],
    "fw_kernels_f32.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    "fw_api.cu": [],
    "fw_init.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "fw_noalloc.cu": ["-fmad=false"],
    "fw_learn.cu": [],
}

FW_ERRORS = {0: "FW_OK", -1: "FW_ERR_CUDA", -2: "FW_ERR_OOM", -3: "FW_ERR_BAD_PARAM",
             -4: "FW_ERR_BLOWUP", -5: "FW_ERR_NAN", -6: "FW_ERR_UNSUPPORTED",
             -7: "FW_ERR_NOT_READY", -8: "FW_ERR_NO_DEVICE", -9: "FW_ERR_IO",
             -10: "FW_ERR_TIMEOUT"}


class FwError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s (%d)%s" % (FW_ERRORS.get(status, "?"), status,
                                        (": " + what) if what else ""))


def lib_path():
    return os.path.join(_BUILD, "libfunwave_gpu.so")


def build(verbose=False):
    """Compile the CUDA library for sm_103a with nvcc (no GPU needed).

    Each translation unit is compiled in parallel, then linked into
    ``_build/libfunwave_gpu.so``.  Rebuilds only when a source is newer."""
    os.makedirs(_BUILD, exist_ok=True)
    out = lib_path()
    srcs = [os.path.join(_CSRC, s) for s in _SOURCES]
    deps = srcs + [os.path.join(_CSRC, h) for h in os.listdir(_CSRC)
                   if h.endswith(".h") or h.endswith(".cuh")] + [_HEADER]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        build_driver()
        return out
    nvcc = os.environ.get("NVCC", "nvcc")
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I" + os.path.join(_ROOT, "include")]
    arch = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo"]
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(_BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        cmd = [nvcc] + common + arch + _SOURCES[os.path.basename(s)] + ["-c", s, "-o", o]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        txt = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), txt))
        if verbose and txt.strip():
            print(txt)
    link = [nvcc] + arch + ["-shared", "-o", out + ".tmp"] + objs
    subprocess.run(link, check=True)
    os.replace(out + ".tmp", out)
    build_driver()
    return out


def driver_path():
    return os.path.join(_BUILD, "fw_main")


def build_driver():
    """Compile the C++ host driver (host/fw_main.cpp) against the library."""
    src = os.path.join(_HERE, "host", "fw_main.cpp")
    exe = driver_path()
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(src), os.path.getmtime(lib_path())):
        return exe
    cxx = os.environ.get("CXX", "g++")
    # no fused multiply-adds in host arithmetic: the same files on x86 and Arm
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-pthread", "-ffp-contract=off", "-I" + os.path.join(_ROOT, "include"),
           src, "-L" + _BUILD,
           "-lfunwave_gpu", "-Wl,-rpath,$ORIGIN", "-o", exe + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(exe + ".tmp", exe)
    return exe


class FwParams(ctypes.Structure):
    _fields_ = [
        ("Mglob", ctypes.c_int), ("Nglob", ctypes.c_int),
        ("DX", ctypes.c_double), ("DY", ctypes.c_double),
        ("periodic", ctypes.c_int), ("dispersion", ctypes.c_int),
        ("gamma1", ctypes.c_double), ("gamma2", ctypes.c_double),
        ("gamma3", ctypes.c_double), ("beta_ref", ctypes.c_double),
        ("viscosity_breaking", ctypes.c_int), ("show_breaking", ctypes.c_int),
        ("cbrk1", ctypes.c_double), ("cbrk2", ctypes.c_double),
        ("wavemaker_cbrk", ctypes.c_double), ("nu_bkg", ctypes.c_double),
        ("swe_eta_dep", ctypes.c_double), ("cfl", ctypes.c_double),
        ("fixed_dt", ctypes.c_int), ("dt_fixed", ctypes.c_double),
        ("froude_cap", ctypes.c_double), ("min_depth", ctypes.c_double),
        ("min_depth_frc", ctypes.c_double), ("eta_limiter", ctypes.c_int),
        ("trough_limit", ctypes.c_double), ("crest_limit", ctypes.c_double),
        ("direct_sponge", ctypes.c_int),
        ("sponge_west", ctypes.c_double), ("sponge_east", ctypes.c_double),
        ("sponge_south", ctypes.c_double), ("sponge_north", ctypes.c_double),
        ("r_sponge", ctypes.c_double), ("a_sponge", ctypes.c_double),
        ("friction_sponge", ctypes.c_int), ("cd_fixed", ctypes.c_double),
        ("wavemaker", ctypes.c_int),
        ("amp_wk", ctypes.c_double), ("tperiod", ctypes.c_double),
        ("dep_wk", ctypes.c_double), ("xc_wk", ctypes.c_double),
        ("yc_wk", ctypes.c_double), ("theta_wk", ctypes.c_double),
        ("delta_wk", ctypes.c_double), ("time_ramp", ctypes.c_double),
        ("ywidth_wk", ctypes.c_double),
        ("freq_peak", ctypes.c_double), ("freq_min", ctypes.c_double),
        ("freq_max", ctypes.c_double), ("gamma_tma", ctypes.c_double),
        ("hmo", ctypes.c_double), ("theta_peak", ctypes.c_double),
        ("sigma_theta", ctypes.c_double),
        ("nfreq", ctypes.c_int), ("ntheta", ctypes.c_int),
        ("spreading", ctypes.c_int), ("spread_s", ctypes.c_double),
        ("precision", ctypes.c_int), ("device", ctypes.c_int),
        ("track_hmax", ctypes.c_int),
        ("track_hmin", ctypes.c_int), ("track_umax", ctypes.c_int), ("track_mfmax", ctypes.c_int),
        ("steady_time", ctypes.c_double), ("t_intv_mean", ctypes.c_double),
        ("track_roller", ctypes.c_int), ("track_radiation", ctypes.c_int),
    ]


_KEYS = {
    "Mglob": "Mglob", "Nglob": "Nglob", "DX": "DX", "DY": "DY",
    "PERIODIC": "periodic", "DISPERSION": "dispersion", "Gamma1": "gamma1",
    "Gamma2": "gamma2", "Gamma3": "gamma3", "Beta_ref": "beta_ref",
    "VISCOSITY_BREAKING": "viscosity_breaking", "SHOW_BREAKING": "show_breaking",
    "Cbrk1": "cbrk1", "Cbrk2": "cbrk2", "WAVEMAKER_Cbrk": "wavemaker_cbrk",
    "nu_bkg": "nu_bkg", "SWE_ETA_DEP": "swe_eta_dep", "CFL": "cfl",
    "DT_fixed": "dt_fixed", "FroudeCap": "froude_cap", "MinDepth": "min_depth",
    "MinDepthFrc": "min_depth_frc", "ETA_LIMITER": "eta_limiter",
    "TroughLimit": "trough_limit", "CrestLimit": "crest_limit",
    "DIRECT_SPONGE": "direct_sponge", "Sponge_west_width": "sponge_west",
    "Sponge_east_width": "sponge_east", "Sponge_south_width": "sponge_south",
    "Sponge_north_width": "sponge_north", "R_sponge": "r_sponge",
    "A_sponge": "a_sponge", "FRICTION_SPONGE": "friction_sponge", "Cd": "cd_fixed",
    "AMP_WK": "amp_wk", "Tperiod": "tperiod", "DEP_WK": "dep_wk", "Xc_WK": "xc_wk",
    "Yc_WK": "yc_wk", "Theta_WK": "theta_wk", "Delta_WK": "delta_wk",
    "Time_ramp": "time_ramp", "Ywidth_WK": "ywidth_wk", "FreqPeak": "freq_peak",
    "FreqMin": "freq_min", "FreqMax": "freq_max", "GammaTMA": "gamma_tma",
    "Hmo": "hmo", "ThetaPeak": "theta_peak", "Sigma_Theta": "sigma_theta",
    "Nfreq": "nfreq", "Ntheta": "ntheta", "SPREADING_S": "spread_s",
    "OUT_Hmax": "track_hmax", "OUT_Hmin": "track_hmin", "OUT_Umax": "track_umax",
    "OUT_MFmax": "track_mfmax", "STEADY_TIME": "steady_time", "T_INTV_mean": "t_intv_mean",
}
_WK = {"NONE": 0, "WK_REG": 1, "JON_2D": 2}


def params_struct(p, precision=None, device=0):
    """Fill FwParams from an input.txt-style dictionary."""
    p = with_defaults(p)
    s = FwParams()
    for k, name in _KEYS.items():
        if k in p:
            t = dict(FwParams._fields_)[name]
            setattr(s, name, int(p[k]) if t is ctypes.c_int else float(p[k]))
    s.fixed_dt = 1 if p.get("DT_fixed", 0) else 0
    if p["WAVEMAKER"] not in _WK:
        raise FwError(-6, "WAVEMAKER=%s is outside the built hot path" % p["WAVEMAKER"])
    s.wavemaker = _WK[p["WAVEMAKER"]]
    s.spreading = 1 if p.get("SPREADING", "WRAPPED_NORMAL") == "COS2S" else 0
    prec = precision or p.get("PRECISION", "FP64")
    s.precision = {"FP64": 0, "MIXED": 1}[prec.upper()]
    s.device = int(device)
    # ROLLER and UNDERTOW (output switches) both need the BREAKING diagnostics
    s.track_roller = 1 if (p.get("ROLLER", False) or p.get("UNDERTOW", False)) else 0
    # PREVIEW_MEAN's Radiation files and the ulagm/vlagm of Umean/Vmean need
    # CALCULATE_MEAN's radiation-stress sums (P_mean, Q_mean among them)
    s.track_radiation = 1 if any(p.get(k, False) for k in ("OUT_Radiation", "OUT_Umean", "OUT_Vmean")) else 0
    return s


_lib = None


def declared_symbols():
    """Function names declared in include/funwave_gpu.h."""
    txt = open(_HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fw_[a-z_0-9]+)\s*\(", txt)))


def load_library(path=None):
    """Load the library (building it first if needed) and declare its ABI."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or lib_path()
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.fw_params_default.argtypes = [ctypes.POINTER(FwParams)]
    L.fw_params_default.restype = None
    L.fw_create.argtypes = [ctypes.POINTER(FwParams), ctypes.POINTER(vp)]
    L.fw_destroy.argtypes = [vp]
    L.fw_init.argtypes = [vp] + [ctypes.POINTER(dp)] * 5
    L.fw_get_field.argtypes = [vp, ctypes.c_char_p, vp]
    L.fw_get_field_f32.argtypes = [vp, ctypes.c_char_p, vp]
    L.fw_set_field_f32.argtypes = [vp, ctypes.c_char_p, vp]
    L.fw_set_field.argtypes = [vp, ctypes.c_char_p, vp]
    L.fw_get_scalar.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(dp)]
    L.fw_set_scalar.argtypes = [vp, ctypes.c_char_p, dp]
    for n in ("begin_step", "exchange", "estimate_dt", "cal_dispersion", "fluxes",
              "source_terms", "update_mask", "wave_breaking", "sponge_damping", "sync"):
        getattr(L, "fw_" + n).argtypes = [vp]
    L.fw_stage.argtypes = [vp, ip]
    L.fw_estimate_huv.argtypes = [vp, ip]
    L.fw_end_step.argtypes = [vp, ctypes.POINTER(ip)]
    L.fw_step.argtypes = [vp, ip, ctypes.POINTER(ip)]
    L.fw_step_async.argtypes = [vp, ip]
    L.fw_get_points.argtypes = [vp, ctypes.c_char_p, ip, ctypes.POINTER(ip), ctypes.POINTER(ip),
                                ctypes.POINTER(dp)]
    L.fw_step_wait.argtypes = [vp, ctypes.POINTER(ip)]
    L.fw_ensemble_step.argtypes = [ctypes.POINTER(vp), ip, ip, ctypes.POINTER(ip)]
    L.fw_ensemble_create.argtypes = [ctypes.POINTER(vp), ip, ctypes.POINTER(vp)]
    L.fw_ensemble_run.argtypes = [vp, ip, ctypes.POINTER(ip)]
    L.fw_ensemble_destroy.argtypes = [vp]
    L.fw_launch_count.argtypes = [vp]
    L.fw_launch_count.restype = ctypes.c_longlong
    L.fw_stream.argtypes = [vp]
    L.fw_stream.restype = vp
    L.fw_time_kernel.argtypes = [vp, ctypes.c_char_p, ip, ctypes.POINTER(dp)]
    L.fw_autotune.argtypes = [vp, ip]
    L.fw_get_tuning.argtypes = [vp, ctypes.POINTER(ip)]
    L.fw_set_tuning.argtypes = [vp, ctypes.POINTER(ip)]
    L.fw_output_begin.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(vp)]
    L.fw_set_fields.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(vp)]
    L.fw_get_fields.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(vp)]
    L.fw_set_fields_f32.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(vp)]
    L.fw_get_fields_f32.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(vp)]
    L.fw_output_wait.argtypes = [vp]
    L.fw_output_done.argtypes = [vp]
    L.fw_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(vp)]
    L.fw_host_free.argtypes = [vp]
    L.fw_checkpoint.argtypes = [vp, ctypes.c_char_p]
    L.fw_restore.argtypes = [vp, ctypes.c_char_p]
    L.fw_strerror.argtypes = [ip]
    L.fw_strerror.restype = ctypes.c_char_p
    if path == lib_path():
        _lib = L
    return L


_MASKS = {"MASK", "MASK9", "MASK_STRUC"}
_XFACE = {"Depthx", "P", "Fx", "Gx"}
_YFACE = {"Depthy", "Q", "Fy", "Gy"}


def _dptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Solver:
    """One device-resident FUNWAVE-TVD case."""

    def __init__(self, params, precision=None, device=0):
        self.params = with_defaults(params)
        self.L = load_library()
        self._p = params_struct(self.params, precision, device)
        h = ctypes.c_void_p()
        self._check(self.L.fw_create(ctypes.byref(self._p), ctypes.byref(h)), "fw_create")
        self.ctx = h
        self.Mloc = self._p.Mglob + 6
        self.Nloc = self._p.Nglob + 6
        self.precision = "FP64" if self._p.precision == 0 else "MIXED"

    def _check(self, rc, what=""):
        if rc != 0:
            raise FwError(rc, what)

    def close(self):
        if getattr(self, "ctx", None):
            self.L.fw_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- set-up ---------------------------------------------------------
    def init(self, depth, eta=None, u=None, v=None, phases=None):
        """INITIALIZATION from interior arrays (Mglob x Nglob, x first)."""
        def f(a):
            return None if a is None else np.asfortranarray(np.asarray(a, dtype=np.float64))
        d, e, uu, vv = f(depth), f(eta), f(u), f(v)
        ph = f(phases)
        self._keep = (d, e, uu, vv, ph)
        self._check(self.L.fw_init(self.ctx, _dptr(d), _dptr(e), _dptr(uu), _dptr(vv), _dptr(ph)),
                    "fw_init")

    # --- fields ---------------------------------------------------------
    def shape(self, name):
        if name in _XFACE:
            return (self.Mloc + 1, self.Nloc)
        if name in _YFACE:
            return (self.Mloc, self.Nloc + 1)
        return (self.Mloc, self.Nloc)

    def get(self, name):
        dt = np.int32 if name in _MASKS else np.float64
        a = np.zeros(self.shape(name), dtype=dt, order="F")
        self._check(self.L.fw_get_field(self.ctx, name.encode(), a.ctypes.data), "get " + name)
        return a

    def get_f32(self, name):
        """A field as float32 (fw_get_field_f32: the REAL(SP) host arrays of
        a single-precision build)."""
        a = np.zeros(self.shape(name), dtype=np.float32, order="F")
        self._check(self.L.fw_get_field_f32(self.ctx, name.encode(), a.ctypes.data), "get_f32 " + name)
        return a

    def set_f32(self, name, arr):
        a = np.asfortranarray(np.asarray(arr, dtype=np.float32))
        if a.shape != self.shape(name):
            raise FwError(-3, "%s must have shape %s" % (name, self.shape(name)))
        self._check(self.L.fw_set_field_f32(self.ctx, name.encode(), a.ctypes.data), "set_f32 " + name)

    def set(self, name, arr):
        dt = np.int32 if name in _MASKS else np.float64
        a = np.asfortranarray(np.asarray(arr, dtype=dt))
        if a.shape != self.shape(name):
            raise FwError(-3, "%s must have shape %s" % (name, self.shape(name)))
        self._check(self.L.fw_set_field(self.ctx, name.encode(), a.ctypes.data), "set " + name)

    def set_fields(self, arrays):
        """{name: array} to the device in one call (fw_set_fields); arrays in
        the layout of set() (Fortran-ordered float64, int32 for masks)."""
        names = list(arrays)
        keep = []
        for n in names:
            dt = np.int32 if n in _MASKS else np.float64
            a = np.asfortranarray(arrays[n], dtype=dt)
            if a.shape != self.shape(n):
                raise ValueError("%s: shape %s, expected %s" % (n, a.shape, self.shape(n)))
            keep.append(a)
        cn = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
        hp = (ctypes.c_void_p * len(names))(*[a.ctypes.data for a in keep])
        self._check(self.L.fw_set_fields(self.ctx, len(names), cn, hp), "fw_set_fields")

    def get_fields(self, names):
        """{name: array} from the device in one call (fw_get_fields)."""
        names = list(names)
        out = {n: np.zeros(self.shape(n), dtype=np.int32 if n in _MASKS else np.float64, order="F") for n in names}
        cn = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
        hp = (ctypes.c_void_p * len(names))(*[out[n].ctypes.data for n in names])
        self._check(self.L.fw_get_fields(self.ctx, len(names), cn, hp), "fw_get_fields")
        return out

    def __getitem__(self, name):
        return self.get(name)

    def scalar(self, name):
        v = ctypes.c_double()
        self._check(self.L.fw_get_scalar(self.ctx, name.encode(), ctypes.byref(v)), name)
        return v.value

    def set_scalar(self, name, value):
        self._check(self.L.fw_set_scalar(self.ctx, name.encode(), float(value)), name)

    # --- time stepping (main.F:284-535) ---------------------------------
    def step(self, nsteps=1, check=True):
        st = ctypes.c_int()
        self._check(self.L.fw_step(self.ctx, int(nsteps), ctypes.byref(st)), "fw_step")
        if check and st.value != 0:
            raise FwError(st.value, "after %d steps" % nsteps)
        return st.value

    def step_async(self, nsteps=1):
        """Enqueue nsteps whole steps and return at once (fw_step_async)."""
        self._check(self.L.fw_step_async(self.ctx, int(nsteps)), "fw_step_async")

    def step_wait(self, check=True):
        """Wait for the steps of step_async; their CHECK_BLOWUP status."""
        st = ctypes.c_int()
        self._check(self.L.fw_step_wait(self.ctx, ctypes.byref(st)), "fw_step_wait")
        if check and st.value != 0:
            raise FwError(st.value, "after step_async")
        return st.value

    def begin_step(self):
        self._check(self.L.fw_begin_step(self.ctx), "fw_begin_step")

    def stage(self, istage):
        self._check(self.L.fw_stage(self.ctx, int(istage)), "fw_stage")

    def end_step(self):
        st = ctypes.c_int()
        self._check(self.L.fw_end_step(self.ctx, ctypes.byref(st)), "fw_end_step")
        return st.value

    def sync(self):
        self._check(self.L.fw_sync(self.ctx), "fw_sync")

    # --- asynchronous output ---------------------------------------------
    def output_begin(self, names):
        """Snapshot the named fields after the steps enqueued so far and copy
        them to pinned host buffers while later steps run (fw_output_begin).
        Returns an :class:`Output`; its wait() gives {name: array} as get()
        would.  A later output_begin first waits for this one's copies."""
        return Output(self, list(names))

    # --- restart ----------------------------------------------------------
    def checkpoint(self, path):
        """Write the complete run state to path (fw_checkpoint)."""
        self._check(self.L.fw_checkpoint(self.ctx, os.fsencode(path)), "fw_checkpoint")

    def restore(self, path):
        """Load a checkpoint written by a Solver with the same parameters;
        no init() is needed first (fw_restore).  The run then continues bit
        for bit as the checkpointed one."""
        self._check(self.L.fw_restore(self.ctx, os.fsencode(path)), "fw_restore")

    # --- the reference's units ------------------------------------------
    def exchange(self):
        self._check(self.L.fw_exchange(self.ctx), "EXCHANGE")

    def estimate_dt(self):
        self._check(self.L.fw_estimate_dt(self.ctx), "ESTIMATE_DT")

    def cal_dispersion(self):
        self._check(self.L.fw_cal_dispersion(self.ctx), "CAL_DISPERSION")

    def fluxes(self):
        self._check(self.L.fw_fluxes(self.ctx), "FLUXES")

    def source_terms(self):
        self._check(self.L.fw_source_terms(self.ctx), "SourceTerms")

    def estimate_huv(self, istage):
        self._check(self.L.fw_estimate_huv(self.ctx, int(istage)), "ESTIMATE_HUV")

    def update_mask(self):
        self._check(self.L.fw_update_mask(self.ctx), "UPDATE_MASK")

    def wave_breaking(self):
        self._check(self.L.fw_wave_breaking(self.ctx), "WAVE_BREAKING")

    def sponge_damping(self):
        self._check(self.L.fw_sponge_damping(self.ctx), "SPONGE_DAMPING")

    def time_kernel(self, name, nrep=20):
        """Average duration (ms) of one kernel of the step, CUDA events."""
        ms = ctypes.c_double()
        self._check(self.L.fw_time_kernel(self.ctx, name.encode(), int(nrep), ctypes.byref(ms)), name)
        return ms.value

    # FW_TUNE_LEN of include/funwave_gpu.h: (bx, by) of disp_a, disp_b,
    # update, post_mask_break, maskmul, then the x and y flux tile heights
    TUNE_LEN = 14
    TUNE_NAMES = ("disp_a", "disp_b", "update", "post_mask_break", "maskmul")

    def autotune(self, fresh=False):
        """Time the candidate launch shapes on this run's state (saved and
        restored around the measurement) and keep the fastest; returns the
        tuning (see tuning())."""
        self._check(self.L.fw_autotune(self.ctx, 1 if fresh else 0), "fw_autotune")
        return self.tuning()

    def tuning(self):
        """{kernel: (bx, by)} of the per-cell kernels plus "flux_x"/"flux_y"
        tile heights."""
        t = (ctypes.c_int * self.TUNE_LEN)()
        self._check(self.L.fw_get_tuning(self.ctx, t), "fw_get_tuning")
        out = {n: (t[2 * k], t[2 * k + 1]) for k, n in enumerate(self.TUNE_NAMES)}
        out["flux_x"], out["flux_y"] = t[10], t[11]
        out["flux_x_tma"], out["flux_y_tma"] = t[12], t[13]
        return out

    def set_tuning(self, tuning):
        """Set launch shapes explicitly (a dict as returned by tuning())."""
        t = (ctypes.c_int * self.TUNE_LEN)()
        for k, n in enumerate(self.TUNE_NAMES):
            t[2 * k], t[2 * k + 1] = tuning[n]
        t[10], t[11] = tuning["flux_x"], tuning["flux_y"]
        # TMA staging of the flux tiles; 0 (each thread loads) when not given
        t[12], t[13] = tuning.get("flux_x_tma", 0), tuning.get("flux_y_tma", 0)
        self._check(self.L.fw_set_tuning(self.ctx, t), "fw_set_tuning")

    def launch_count(self):
        return int(self.L.fw_launch_count(self.ctx))

    def stream(self):
        return self.L.fw_stream(self.ctx)


class Output:
    """The pinned host buffers of one fw_output_begin (Solver.output_begin)."""

    def __init__(self, solver, names):
        self.s, self.names = solver, names
        self.arrays, self._ptrs = {}, []
        self._seq = None
        L = solver.L
        try:
            for n in names:
                shape = solver.shape(n)
                dt = np.int32 if n in _MASKS else np.float64
                nbytes = int(np.prod(shape)) * np.dtype(dt).itemsize
                p = ctypes.c_void_p()
                solver._check(L.fw_host_alloc(nbytes, ctypes.byref(p)), "fw_host_alloc")
                self._ptrs.append(p.value)
                buf = (ctypes.c_char * nbytes).from_address(p.value)
                self.arrays[n] = np.frombuffer(buf, dtype=dt).reshape(shape, order="F")
            cn = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
            hp = (ctypes.c_void_p * len(names))(*self._ptrs)
            solver._check(L.fw_output_begin(solver.ctx, len(names), cn, hp), "fw_output_begin")
            # a later fw_output_begin waits for this one's copies first
            solver._out_seq = getattr(solver, "_out_seq", 0) + 1
            self._seq = solver._out_seq
        except Exception:
            self._free()
            raise

    def _superseded(self):
        return self._seq != self.s._out_seq

    def done(self):
        if self._superseded():
            return True
        rc = self.s.L.fw_output_done(self.s.ctx)
        if rc < 0:
            raise FwError(rc, "fw_output_done")
        return rc == 1

    def wait(self):
        """Wait for the copies; returns {name: array} (copies of the pinned
        buffers, which are then released)."""
        if not self._superseded():
            self.s._check(self.s.L.fw_output_wait(self.s.ctx), "fw_output_wait")
        out = {n: a.copy() for n, a in self.arrays.items()}
        self._free()
        return out

    def _free(self):
        self.arrays = {}
        for p in self._ptrs:
            self.s.L.fw_host_free(p)
        self._ptrs = []

    def __del__(self):
        try:
            if self._ptrs:
                if not self._superseded():
                    self.s.L.fw_output_wait(self.s.ctx)
                self._free()
        except Exception:
            pass
