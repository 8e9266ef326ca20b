"""input.txt parameters of the hot path.

Key names and defaults follow the reference's READ_INPUT (src/io.F:149-3773,
the READ_* call sites and their "Default" branches).  Parsing follows
READ_VALUE (src/mod_input.F:271-308): a line is ``KEY = value``, anything
after ``!`` is a comment, the first line whose key matches wins, and logical
values are ``T``/``F`` (Fortran list-directed input).
"""
import os

# (key, default).  None = no default (the reference stops when missing).
PARAM_DEFAULTS = {
    "Mglob": None, "Nglob": None, "DX": None, "DY": None,
    "DEPTH_TYPE": "DATA", "DEPTH_FILE": "depth.txt", "DEPTH_FLAT": 10.0,
    "SLP": 0.0, "Xslp": 0.0,
    "TOTAL_TIME": 0.0, "PLOT_INTV": 1.0, "SCREEN_INTV": 1.0,
    "PERIODIC": False,
    "DISPERSION": True, "Gamma1": 1.0, "Gamma2": 1.0, "Gamma3": 1.0,
    "Beta_ref": -0.531,
    "VISCOSITY_BREAKING": True, "SHOW_BREAKING": True,
    "Cbrk1": 0.65, "Cbrk2": 0.35, "WAVEMAKER_Cbrk": 1.0, "nu_bkg": 0.0,
    "SWE_ETA_DEP": 0.80,
    "CFL": 0.5, "DT_fixed": 0.0,
    "FroudeCap": 3.0, "MinDepth": 0.1, "MinDepthFrc": 0.1,
    "ETA_LIMITER": False, "TroughLimit": -999999.0, "CrestLimit": 999999.0,
    "DIRECT_SPONGE": False, "FRICTION_SPONGE": False,
    "Sponge_west_width": 0.0, "Sponge_east_width": 0.0,
    "Sponge_south_width": 0.0, "Sponge_north_width": 0.0,
    "R_sponge": 0.85, "A_sponge": 5.0,
    "Cd": 0.0,
    "WAVEMAKER": "NONE",
    "AMP_WK": 0.0, "Tperiod": 0.0, "DEP_WK": 0.0, "Xc_WK": 0.0, "Yc_WK": 0.0,
    "Theta_WK": 0.0, "Delta_WK": 0.5, "Time_ramp": 0.0, "Ywidth_WK": 999999.0,
    "FreqPeak": 0.0, "FreqMin": 0.0, "FreqMax": 0.0, "GammaTMA": 3.3,
    "Hmo": 0.0, "ThetaPeak": 0.0, "Sigma_Theta": 10.0, "Nfreq": 0, "Ntheta": 1,
    # build-side options of this library (not reference keys)
    "SPREADING": "WRAPPED_NORMAL", "SPREADING_S": 10.0,
    "PRECISION": "FP64", "OUT_Hmax": False,
    # statistics (MAX_MIN_PROPERTY switches, MIXING_STUFF times)
    "OUT_Hmin": False, "OUT_Umax": False, "OUT_MFmax": False, "ROLLER": False, "UNDERTOW": False,
    "STEADY_TIME": 999999.0, "T_INTV_mean": 999999.0,
    # PREVIEW_MEAN's files (io.F:4666-4733)
    "OUT_Umean": False, "OUT_Vmean": False, "OUT_ETAmean": False, "OUT_WaveHeight": False,
    "OUT_Radiation": False,
}

# input.txt keys of the output switches (io.F:3392-3424) -> the OUT_*
# variable names this package uses; either spelling is accepted
REFERENCE_KEYS = {
    "Hmax": "OUT_Hmax", "Hmin": "OUT_Hmin", "Umax": "OUT_Umax", "MFmax": "OUT_MFmax", "Umean": "OUT_Umean",
    "Vmean": "OUT_Vmean", "ETAmean": "OUT_ETAmean", "WaveHeight": "OUT_WaveHeight", "Radiation": "OUT_Radiation",
}

_BOOL = {k for k, v in PARAM_DEFAULTS.items() if isinstance(v, bool)}
_INT = {"Mglob", "Nglob", "Nfreq", "Ntheta"}
_STR = {"DEPTH_TYPE", "DEPTH_FILE", "WAVEMAKER", "SPREADING", "PRECISION"}


def with_defaults(p):
    """A copy of p with every missing key set to its reference default."""
    out = {k: v for k, v in PARAM_DEFAULTS.items() if v is not None}
    out.update(p)
    for k in ("Mglob", "Nglob", "DX", "DY"):
        if out.get(k) is None:
            raise ValueError("%s is required (no default in the reference)" % k)
    return out


def _convert(key, text):
    t = text.strip()
    if key in _BOOL:
        u = t.upper().lstrip(".")
        if u.startswith("T"):
            return True
        if u.startswith("F"):
            return False
        raise ValueError("bad logical for %s: %r" % (key, text))
    if key in _INT:
        return int(float(t))
    if key in _STR:
        return t.split()[0] if t else t
    try:
        return float(t.replace("d", "e").replace("D", "e"))
    except ValueError:
        return t


def read_input_txt(path_or_text):
    """Parse an input.txt (path or text) into a dictionary of known keys.

    Unknown keys are kept as strings under their own name.  As in
    READ_VALUE, only the first occurrence of a key counts."""
    if os.path.exists(str(path_or_text)):
        with open(path_or_text) as fh:
            text = fh.read()
    else:
        text = str(path_or_text)
    out = {}
    for line in text.splitlines():
        body = line.split("!", 1)[0]
        if "=" not in body:
            continue
        key, val = body.split("=", 1)
        key = key.strip()
        key = REFERENCE_KEYS.get(key, key)
        if not key or key in out:
            continue
        out[key] = _convert(key, val)
    return out
