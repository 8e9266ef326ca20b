"""ctypes driver for the C oracle (oracle/fw_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py``.  The product never imports it.

``Oracle(params)`` takes the same parameter dictionary as the product's host
layer (input.txt key names, see ``funwave_gpu.PARAM_DEFAULTS``) and exposes
the oracle's arrays as Fortran-ordered numpy views with the reference's
extents (ghost cells included).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfw_oracle.so")
_LIB32_PATH = os.path.join(_HERE, "_build", "libfw_oracle_f32.so")


class OfwParams(ctypes.Structure):
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
        ("track_hmax", ctypes.c_int), ("track_hmin", ctypes.c_int), ("track_umax", ctypes.c_int),
        ("track_mfmax", ctypes.c_int), ("steady_time", ctypes.c_double), ("t_intv_mean", ctypes.c_double),
    ]


# input.txt key -> oracle field
_KEYMAP = {
    "Mglob": "Mglob", "Nglob": "Nglob", "DX": "DX", "DY": "DY",
    "PERIODIC": "periodic", "DISPERSION": "dispersion",
    "Gamma1": "gamma1", "Gamma2": "gamma2", "Gamma3": "gamma3",
    "Beta_ref": "beta_ref", "VISCOSITY_BREAKING": "viscosity_breaking",
    "SHOW_BREAKING": "show_breaking", "Cbrk1": "cbrk1", "Cbrk2": "cbrk2",
    "WAVEMAKER_Cbrk": "wavemaker_cbrk", "nu_bkg": "nu_bkg",
    "SWE_ETA_DEP": "swe_eta_dep", "CFL": "cfl", "DT_fixed": "dt_fixed",
    "FroudeCap": "froude_cap", "MinDepth": "min_depth",
    "MinDepthFrc": "min_depth_frc", "ETA_LIMITER": "eta_limiter",
    "TroughLimit": "trough_limit", "CrestLimit": "crest_limit",
    "DIRECT_SPONGE": "direct_sponge", "Sponge_west_width": "sponge_west",
    "Sponge_east_width": "sponge_east", "Sponge_south_width": "sponge_south",
    "Sponge_north_width": "sponge_north", "R_sponge": "r_sponge",
    "A_sponge": "a_sponge", "FRICTION_SPONGE": "friction_sponge",
    "Cd": "cd_fixed", "AMP_WK": "amp_wk", "Tperiod": "tperiod",
    "DEP_WK": "dep_wk", "Xc_WK": "xc_wk", "Yc_WK": "yc_wk",
    "Theta_WK": "theta_wk", "Delta_WK": "delta_wk", "Time_ramp": "time_ramp",
    "Ywidth_WK": "ywidth_wk", "FreqPeak": "freq_peak", "FreqMin": "freq_min",
    "FreqMax": "freq_max", "GammaTMA": "gamma_tma", "Hmo": "hmo",
    "ThetaPeak": "theta_peak", "Sigma_Theta": "sigma_theta", "Nfreq": "nfreq",
    "Ntheta": "ntheta", "SPREADING_S": "spread_s",
    "OUT_Hmax": "track_hmax", "OUT_Hmin": "track_hmin", "OUT_Umax": "track_umax",
    "OUT_MFmax": "track_mfmax", "STEADY_TIME": "steady_time", "T_INTV_mean": "t_intv_mean",
}
_WAVEMAKERS = {"NONE": 0, "WK_REG": 1, "JON_2D": 2}


def build():
    """Compile the oracle library with its Makefile (gcc, no GPU needed)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_libs = {}


def lib(fp32=False):
    """The FP64 oracle (the checker), or with fp32 its single-precision build
    (timed only, as the CPU baseline of a REAL(SP) = 4-byte reference build)."""
    if fp32 not in _libs:
        path = _LIB32_PATH if fp32 else _LIB_PATH
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.ofw_create.restype = vp
        L.ofw_create.argtypes = [ctypes.POINTER(OfwParams)]
        L.ofw_destroy.argtypes = [vp]
        L.ofw_field.restype = vp
        L.ofw_field.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(ctypes.c_int)]
        L.ofw_get_scalar.restype = ctypes.c_double
        L.ofw_get_scalar.argtypes = [vp, ctypes.c_char_p]
        L.ofw_set_scalar.argtypes = [vp, ctypes.c_char_p, ctypes.c_double]
        L.ofw_init.argtypes = [vp]
        L.ofw_init.restype = ctypes.c_int
        L.ofw_set_phases.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        for n in ("omega", "cm", "sm", "dgen", "rlamda", "betagen"):
            f = getattr(L, "ofw_jon_" + n)
            f.restype = ctypes.POINTER(ctypes.c_double)
            f.argtypes = [vp]
        L.ofw_step.argtypes = [vp]
        L.ofw_step.restype = ctypes.c_int
        for n in ("exchange", "estimate_dt", "cal_dispersion", "fluxes", "source_terms",
                  "update_mask", "wave_breaking", "sponge_damping", "begin_step",
                  "max_min_property", "mixing_stuff"):
            getattr(L, "ofw_" + n).argtypes = [vp]
        L.ofw_estimate_huv.argtypes = [vp, ctypes.c_int]
        L.ofw_stage.argtypes = [vp, ctypes.c_int]
        L.ofw_check_blowup.argtypes = [vp]
        L.ofw_check_blowup.restype = ctypes.c_int
        L.ofw_end_step.argtypes = [vp]
        L.ofw_end_step.restype = ctypes.c_int
        L.ofw_set_threads.argtypes = [ctypes.c_int]
        L.ofw_get_threads.restype = ctypes.c_int
        L.ofw_real_bytes.restype = ctypes.c_int
        _libs[fp32] = L
    return _libs[fp32]


def make_params(p):
    """Fill an OfwParams from an input.txt-style dictionary (defaults applied
    by the caller)."""
    s = OfwParams()
    s.steady_time = 999999.0   # STEADY_TIME and T_INTV_mean default to LARGE
    s.t_intv_mean = 999999.0
    for k, v in p.items():
        if k in _KEYMAP:
            name = _KEYMAP[k]
            ftype = dict(OfwParams._fields_)[name]
            setattr(s, name, int(v) if ftype is ctypes.c_int else float(v))
    s.fixed_dt = 1 if p.get("DT_fixed", 0) else 0
    s.wavemaker = _WAVEMAKERS[p.get("WAVEMAKER", "NONE")]
    s.spreading = 1 if p.get("SPREADING", "WRAPPED_NORMAL") == "COS2S" else 0
    return s


class Oracle:
    def __init__(self, params, threads=0, fp32=False):
        self.params = dict(params)
        self._p = make_params(self.params)
        self.L = lib(fp32)
        self.real = np.float32 if self.L.ofw_real_bytes() == 4 else np.float64
        if threads:
            self.L.ofw_set_threads(int(threads))
        self.ctx = self.L.ofw_create(ctypes.byref(self._p))
        if not self.ctx:
            raise MemoryError("oracle allocation failed")
        self.Mloc = self._p.Mglob + 6
        self.Nloc = self._p.Nglob + 6

    def close(self):
        if self.ctx:
            self.L.ofw_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, kind):
        return {0: (self.Mloc, self.Nloc), 1: (self.Mloc + 1, self.Nloc),
                2: (self.Mloc, self.Nloc + 1)}[kind]

    def field(self, name):
        kind = ctypes.c_int()
        isint = ctypes.c_int()
        ptr = self.L.ofw_field(self.ctx, name.encode(), ctypes.byref(kind), ctypes.byref(isint))
        if not ptr:
            raise KeyError(name)
        m, n = self.shape(kind.value)
        dt = np.int32 if isint.value else self.real
        buf = (ctypes.c_char * (m * n * np.dtype(dt).itemsize)).from_address(ptr)
        return np.frombuffer(buf, dtype=dt).reshape((m, n), order="F")

    def __getitem__(self, name):
        return self.field(name)

    def scalar(self, name):
        return self.L.ofw_get_scalar(self.ctx, name.encode())

    def set_scalar(self, name, v):
        self.L.ofw_set_scalar(self.ctx, name.encode(), float(v))

    def set_phases(self, phases):
        ph = np.ascontiguousarray(np.asarray(phases, dtype=np.float64).ravel(order="F"))
        self.L.ofw_set_phases(self.ctx, ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def init(self):
        rc = self.L.ofw_init(self.ctx)
        if rc != 0:
            raise RuntimeError("oracle init failed (%d)" % rc)

    def band(self):
        return tuple(int(self.scalar(k)) for k in ("ilo", "ihi", "jlo", "jhi"))

    def jon_tables(self):
        nf, nt = self._p.nfreq, self._p.ntheta
        ilo, ihi, jlo, jhi = self.band()
        nb = max(ihi - ilo + 1, 0) * max(jhi - jlo + 1, 0) * nf

        def arr(f, n):
            p = f(self.ctx)
            return np.ctypeslib.as_array(p, shape=(n,)).copy() if p and n else np.zeros(0)
        L = self.L
        return {
            "omega": arr(L.ofw_jon_omega, nf),
            "cm": arr(L.ofw_jon_cm, nb),
            "sm": arr(L.ofw_jon_sm, nb),
            "dgen": arr(L.ofw_jon_dgen, nf * nt),
            "rlamda": arr(L.ofw_jon_rlamda, nf * nt),
            "betagen": arr(L.ofw_jon_betagen, nf),
        }

    def step(self):
        return self.L.ofw_step(self.ctx)

    def begin_step(self):
        self.L.ofw_begin_step(self.ctx)

    def end_step(self):
        return self.L.ofw_end_step(self.ctx)

    def stage(self, istage):
        self.L.ofw_stage(self.ctx, int(istage))

    def call(self, name, *args):
        getattr(self.L, "ofw_" + name)(self.ctx, *args)
