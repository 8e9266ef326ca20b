"""Seeded synthetic cases with the shapes of the benchmark configurations.

The reference measures on no public dataset; these generators stand in for
its input decks.  Each returns ``(params, depth, phases)``: an input.txt-style
dictionary, the interior depth (Mglob x Nglob, x = cross-shore first, metres,
positive down) and the JON_2D phases (or None).

  planar_beach   2-D planar beach with a regular wavemaker and a west
                 sponge, periodic in y (the 250 x 500 configuration)
  shoal_jonswap  1:50 slope from 20 m with an elliptic shoal and a
                 directional JONSWAP wavemaker (the 2048 x 2048 configuration)
  barred_beach   1:40 slope with a Gaussian bar cut by rip channels and a
                 normal-incidence JONSWAP wavemaker (the 4096 x 4096
                 precision configuration)
  ensemble_members  planar beaches of uneven grid size, slope, depth and
                 JONSWAP forcing (the 512-run ensemble configuration)
"""
import numpy as np


def _smooth(noise, sigma_cells, periodic_y):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(noise, sigma=sigma_cells, mode=("nearest", "wrap" if periodic_y else "nearest"))


def planar_beach(Mglob=250, Nglob=500, dx=1.0, seed=0, noise_std=0.02, noise_sigma=5.0,
                 **overrides):
    """Depth 5 m for x < 100 m, then a 1:20 slope up to 2 m above still water,
    plus a seeded N(0, noise_std) field smoothed by a Gaussian of standard
    deviation noise_sigma metres and rescaled back to noise_std.  WK_REG
    H = 0.3 m, T = 6 s at x = 50 m (Time_ramp = 1 period), 30 m west sponge,
    periodic in y, MinDepth 0.01 m, other keys at their reference defaults."""
    x = np.arange(Mglob) * dx
    h = np.where(x < 100.0, 5.0, 5.0 - (x - 100.0) / 20.0)
    h = np.maximum(h, -2.0)
    depth = np.repeat(h[:, None], Nglob, axis=1)
    if noise_std > 0:
        rng = np.random.default_rng(seed)
        n = rng.normal(0.0, noise_std, size=(Mglob, Nglob))
        n = _smooth(n, noise_sigma / dx, True)
        s = n.std()
        if s > 0:
            n = n * (noise_std / s)
        depth = depth + n
    p = {
        "Mglob": Mglob, "Nglob": Nglob, "DX": dx, "DY": dx,
        "PERIODIC": True, "WAVEMAKER": "WK_REG",
        "AMP_WK": 0.15, "Tperiod": 6.0, "DEP_WK": 5.0, "Xc_WK": 50.0,
        "Theta_WK": 0.0, "Delta_WK": 0.5, "Time_ramp": 1.0,
        "DIRECT_SPONGE": True, "Sponge_west_width": 30.0,
        "R_sponge": 0.85, "A_sponge": 5.0,
        "DISPERSION": True, "Gamma1": 1.0, "Gamma2": 1.0, "Gamma3": 1.0,
        "Beta_ref": -0.531, "VISCOSITY_BREAKING": True, "SHOW_BREAKING": True,
        "Cbrk1": 0.65, "Cbrk2": 0.35, "CFL": 0.5,
        "MinDepth": 0.01, "MinDepthFrc": 0.1, "TOTAL_TIME": 300.0,
    }
    p.update(overrides)
    return p, np.asfortranarray(depth), None


def shoal_jonswap(Mglob=2048, Nglob=2048, dx=2.0, seed=0, **overrides):
    """20 m flat offshore, then a 1:50 slope through the shoreline (which
    lies 200 m from the east wall); an elliptic shoal cap
    8*sqrt(1-(dx/200)^2-(dy/150)^2) m high centred 1.5 km offshore of the
    shoreline and mid-domain alongshore.  JON_2D Hs = 1 m, Tp = 10 s,
    gamma = 3.3, 0.05-0.30 Hz in 50 frequencies x 30 directions, cos^2s
    spreading with s = 10, phases uniform on [0, 2pi) from the seed;
    wavemaker at x = 200 m, 100 m west sponge, walls elsewhere."""
    x = np.arange(Mglob) * dx
    y = np.arange(Nglob) * dx
    L = Mglob * dx
    x_shore = L - 200.0
    x_toe = x_shore - 20.0 * 50.0
    h = np.where(x < x_toe, 20.0, 20.0 - (x - x_toe) / 50.0)
    depth = np.repeat(h[:, None], Nglob, axis=1)
    xc, yc = x_shore - 1500.0, y.mean()
    X, Y = np.meshgrid(x, y, indexing="ij")
    r2 = ((X - xc) / 200.0) ** 2 + ((Y - yc) / 150.0) ** 2
    depth = depth - 8.0 * np.sqrt(np.maximum(0.0, 1.0 - r2))
    nf, nt = int(overrides.get("Nfreq", 50)), int(overrides.get("Ntheta", 30))
    rng = np.random.default_rng(seed)
    phases = np.asfortranarray(rng.uniform(0.0, 2.0 * np.pi, size=(nf, nt)))
    p = {
        "Mglob": Mglob, "Nglob": Nglob, "DX": dx, "DY": dx,
        "PERIODIC": False, "WAVEMAKER": "JON_2D",
        "Hmo": 1.0, "FreqPeak": 0.1, "FreqMin": 0.05, "FreqMax": 0.30, "GammaTMA": 3.3,
        "Nfreq": nf, "Ntheta": nt, "ThetaPeak": 0.0, "SPREADING": "COS2S", "SPREADING_S": 10.0,
        "DEP_WK": 20.0, "Xc_WK": 200.0, "Delta_WK": 0.5, "Time_ramp": 1.0,
        "DIRECT_SPONGE": True, "Sponge_west_width": 100.0,
        "DISPERSION": True, "VISCOSITY_BREAKING": True, "SHOW_BREAKING": True,
        "CFL": 0.5, "MinDepth": 0.01, "MinDepthFrc": 0.1, "TOTAL_TIME": 600.0,
    }
    p.update(overrides)
    return p, np.asfortranarray(depth), phases


def random_state(Mglob, Nglob, seed=0, eta_amp=0.05, u_amp=0.1, smooth=3.0):
    """Smooth random interior eta, u, v (for unit parity cases)."""
    rng = np.random.default_rng(seed)
    out = []
    for amp in (eta_amp, u_amp, u_amp):
        f = _smooth(rng.normal(size=(Mglob, Nglob)), smooth, False)
        s = np.abs(f).max()
        out.append(np.asfortranarray(f * (amp / s if s > 0 else 0.0)))
    return tuple(out)


def ensemble_members(n=512, seed=0, nfreq=24, ntheta=8, cells_range=(128 * 256, 1024 * 1024)):
    """n planar-beach runs drawn from one seeded stream: interior cells log-
    uniform in cells_range with the cross-shore/alongshore aspect log-uniform
    in [1/2, 2], dx uniform in [1, 4] m, slope uniform in [1/50, 1/10],
    offshore depth uniform in [5, 20] m, JON_2D Hs uniform in [0.5, 3] m but at
    most 0.15 of the depth at the wavemaker (higher waves make the internal
    wavemaker's source region blow up, in the reference's algorithm as
    here), and Tp uniform in [6, 14] s (gamma 3.3, cos^2s spreading s = 10,
    nfreq x ntheta components, phases from the stream).  Depth is
    min(h0, slope * (x_shore - x)) with the shoreline at 85 % of the domain,
    so every run has dry land; the wavemaker sits at 20 % and a west sponge
    covers 10 %.  Returns a list of (params, depth, phases)."""
    rng = np.random.default_rng(seed)
    out = []
    lo, hi = np.log(cells_range[0]), np.log(cells_range[1])
    for _ in range(n):
        cells = float(np.exp(rng.uniform(lo, hi)))
        aspect = float(np.exp(rng.uniform(np.log(0.5), np.log(2.0))))
        M = max(32, int(round(np.sqrt(cells * aspect) / 8.0)) * 8)
        N = max(32, int(round(cells / M / 8.0)) * 8)
        dx = float(rng.uniform(1.0, 4.0))
        slope = float(rng.uniform(1.0 / 50.0, 1.0 / 10.0))
        h0 = float(rng.uniform(5.0, 20.0))
        x_shore = 0.85 * M * dx
        dep_wk = float(min(h0, slope * (x_shore - 0.2 * M * dx)))
        hs = float(rng.uniform(0.5, max(0.5, min(3.0, 0.15 * dep_wk))))
        tp = float(rng.uniform(6.0, 14.0))
        x = (np.arange(M) + 0.5) * dx
        h = np.minimum(h0, slope * (x_shore - x))
        depth = np.asfortranarray(np.repeat(h[:, None], N, axis=1))
        phases = np.asfortranarray(rng.uniform(0.0, 2.0 * np.pi, size=(nfreq, ntheta)))
        p = {
            "Mglob": M, "Nglob": N, "DX": dx, "DY": dx, "PERIODIC": False, "WAVEMAKER": "JON_2D",
            "Hmo": hs, "FreqPeak": 1.0 / tp, "FreqMin": 0.5 / tp, "FreqMax": 3.0 / tp, "GammaTMA": 3.3,
            "Nfreq": nfreq, "Ntheta": ntheta, "ThetaPeak": 0.0, "SPREADING": "COS2S", "SPREADING_S": 10.0,
            "DEP_WK": dep_wk, "Xc_WK": 0.2 * M * dx,
            "Delta_WK": 0.5, "Time_ramp": 1.0, "DIRECT_SPONGE": True, "Sponge_west_width": 0.1 * M * dx,
            "DISPERSION": True, "VISCOSITY_BREAKING": True, "SHOW_BREAKING": True, "CFL": 0.5,
            "MinDepth": 0.01, "MinDepthFrc": 0.1,
        }
        out.append((p, depth, phases))
    return out


def barred_beach(Mglob=4096, Nglob=4096, dx=1.0, seed=0, h_off=12.0, wk_from_shore=180.0, nfreq=32,
                 ntheta=8, shore_from_east=300.0, **overrides):
    """A 1:40 beach whose shoreline lies shore_from_east m from the east wall, seaward of
    it a flat h_off offshore floor; an alongshore-uniform Gaussian bar 1.5 m
    high and 30 m wide (standard deviation 30/2.355 m) centred 80 m offshore
    of the shoreline, cut by 4 rip channels 20 m wide (the bar is removed
    with cosine-tapered edges) at seeded alongshore positions at least 10 %
    of the domain apart.  JON_2D Hs = 1.5 m, Tp = 10 s, gamma 3.3, normal
    incidence (cos^2s, s = 10), nfreq x ntheta components, wavemaker
    wk_from_shore metres offshore of the shoreline, west sponge 100 m.
    Wetting-drying and breaking are on (the defaults)."""
    x = (np.arange(Mglob) + 0.5) * dx
    y = (np.arange(Nglob) + 0.5) * dx
    x_shore = Mglob * dx - shore_from_east
    h = np.minimum(h_off, (x_shore - x) / 40.0)
    X, Y = np.meshgrid(x, y, indexing="ij")
    bar = 1.5 * np.exp(-0.5 * ((X - (x_shore - 80.0)) / (30.0 / 2.355)) ** 2)
    rng = np.random.default_rng(seed)
    Ly = Nglob * dx
    pos = []
    while len(pos) < 4:
        c = float(rng.uniform(0.05 * Ly, 0.95 * Ly))
        if all(abs(c - q) >= 0.1 * Ly for q in pos):
            pos.append(c)
    cut = np.ones_like(Y)
    for c in pos:
        d = np.abs(Y - c)
        cut = np.minimum(cut, np.where(d <= 10.0, 0.0, np.where(d <= 20.0, 0.5 - 0.5 * np.cos(np.pi * (d - 10.0) / 10.0), 1.0)))
    depth = np.asfortranarray(h[:, None] - bar * cut)
    phases = np.asfortranarray(rng.uniform(0.0, 2.0 * np.pi, size=(nfreq, ntheta)))
    x_wk = x_shore - wk_from_shore
    p = {
        "Mglob": Mglob, "Nglob": Nglob, "DX": dx, "DY": dx, "PERIODIC": False, "WAVEMAKER": "JON_2D",
        "Hmo": 1.5, "FreqPeak": 0.1, "FreqMin": 0.05, "FreqMax": 0.30, "GammaTMA": 3.3,
        "Nfreq": nfreq, "Ntheta": ntheta, "ThetaPeak": 0.0, "SPREADING": "COS2S", "SPREADING_S": 10.0,
        "DEP_WK": float(min(h_off, wk_from_shore / 40.0)), "Xc_WK": x_wk, "Delta_WK": 0.5, "Time_ramp": 1.0,
        "DIRECT_SPONGE": True, "Sponge_west_width": 100.0,
        "DISPERSION": True, "VISCOSITY_BREAKING": True, "SHOW_BREAKING": True,
        "CFL": 0.5, "MinDepth": 0.01, "MinDepthFrc": 0.1,
    }
    p.update(overrides)
    return p, depth, phases, pos
