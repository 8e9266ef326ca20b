"""The Berkhoff (1982) elliptic-shoal benchmark of the reference
(benchmarks/car_berkhoff_2d) run through this library, with the wave height
computed the way the reference's postprocessing/calcheight.m does it.

Data come from tests/golden/berkhoff.npz (written by make_berkhoff.py):
the deck's keys, the bathymetry, the reference's own computed wave-height
field and the laboratory transects.

Deck notes:
* CONSTRUCTION = HLLC selects the HLL fluxes in the reference
  (fluxes.F:109 tests CONSTR(1:3) == 'HLL'), which is what this library has.
* The deck switches its 2 m west and east sponges on with SPONGE_ON = T, a
  key this reference version no longer reads (io.F:2285 reads
  DIRECT_SPONGE, default F).  The committed wave heights fall to ~1e-5 m
  inside both sponges, so they were made with the sponge on:
  DIRECT_SPONGE = T here.
"""
import json
import os

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "berkhoff.npz")
G = 3

# calcheight.m: PLOT_INTV 0.02 s frames, 50 per wave (T = 1 s), the wave
# height is the mean over the last 5 waves (frames 1251..1500) of max - min
PLOT_INTV, PER_WAVE, NWAVE, LAST = 0.02, 50, 5, 1500
FIRST = LAST - NWAVE * PER_WAVE + 1

# showheight.m: transects 1-5 across the shoal at I = 280..440 (+4), 6-8
# along it at J = 80, 100, 120 (+1), 1-based; plot coordinates
# x(i) = (i - 264) * 0.05, y(j) = (j - 100) * 0.1 - 0.15; laboratory values
# are amplitudes in mm (height = 2 x amplitude)
XSHIFT, YSHIFT = 4, 1
CROSS_I = (280, 320, 360, 400, 440)
ALONG_J = (80, 100, 120)


def load():
    d = np.load(FIXTURE)
    deck = json.loads(str(d["params"]))
    depth = np.asfortranarray(d["depth_um"] / 1e6)
    return deck, depth, d


def params(fw, deck):
    p = {k: v for k, v in deck.items() if k in fw.PARAM_DEFAULTS}
    p["DIRECT_SPONGE"] = True
    return fw.with_defaults(p)


def run(fw, precision="FP64"):
    """Run the deck to frame LAST; the wave height (Mglob x Nglob, m) and the
    model time of the last frame."""
    return run_refined(fw, 1, precision)


def run_refined(fw, factor, precision="FP64"):
    """The deck on a grid `factor` times finer in both directions (depth
    interpolated bilinearly between the deck's cell centres); the wave
    height averaged back onto the deck's 600 x 200 cells, and the model
    time of the last frame."""
    from scipy.ndimage import map_coordinates
    deck, depth, _ = load()
    p = params(fw, deck)
    M0, N0 = p["Mglob"], p["Nglob"]
    M, N = M0 * factor, N0 * factor
    if factor > 1:
        p.update(Mglob=M, Nglob=N, DX=p["DX"] / factor, DY=p["DY"] / factor)
        xi = (np.arange(M) + 0.5) / factor - 0.5
        yj = (np.arange(N) + 0.5) / factor - 0.5
        X, Y = np.meshgrid(xi, yj, indexing="ij")
        depth = np.asfortranarray(map_coordinates(depth, [X, Y], order=1, mode="nearest"))
    s = fw.Solver(p, precision=precision)
    s.init(depth)
    height = np.zeros((M, N))
    emax = np.full((M, N), -2000.0)
    emin = np.full((M, N), 2000.0)
    plot_count, frame = 0.0, 0
    while frame < LAST:
        s.step(1)
        # io.F:96-98: PLOT_COUNT accumulates DT; a frame when it reaches
        # PLOT_INTV
        plot_count += s.scalar("DT")
        if plot_count < PLOT_INTV:
            continue
        plot_count -= PLOT_INTV
        frame += 1
        if frame < FIRST:
            continue
        eta = s.get("Eta")[G:-G, G:-G]
        np.maximum(emax, eta, out=emax)
        np.minimum(emin, eta, out=emin)
        if (frame - FIRST + 1) % PER_WAVE == 0:
            height += emax - emin
            emax.fill(-2000.0)
            emin.fill(2000.0)
    t = s.scalar("TIME")
    s.close()
    height /= NWAVE
    if factor > 1:
        height = height.reshape(M0, factor, N0, factor).mean(axis=(1, 3))
    return height, t


def compare(height):
    """Agreement with the reference's wave heights and the laboratory data."""
    _, _, d = load()
    href = d["height_ref"].astype(float)
    M, N = href.shape
    out = {}
    # the domain between the wavemaker and the east sponge (x from 5 m to
    # 28 m: I = 101 .. 560)
    r = (slice(100, 560), slice(0, N))
    diff = height[r] - href[r]
    out["rel_rms_vs_reference_model"] = float(np.sqrt(np.mean(diff ** 2)) / np.sqrt(np.mean(href[r] ** 2)))
    out["max_abs_vs_reference_model_m"] = float(np.abs(diff).max())
    out["corr_vs_reference_model"] = float(np.corrcoef(height[r].ravel(), href[r].ravel())[0, 1])
    y = (np.arange(1, N + 1) - 100) * 0.1 - 0.15
    x = (np.arange(1, M + 1) - 260 - XSHIFT) * 0.05
    lab_err, lab_ref, model_err = [], [], []
    for k, i in enumerate(CROSS_I, 1):
        sec = d["sec%d" % k]
        h_lab = 2e-3 * sec[:, 1]
        h_mod = np.interp(sec[:, 0], y, height[i + XSHIFT - 1, :])
        h_rm = np.interp(sec[:, 0], y, href[i + XSHIFT - 1, :])
        lab_err.append(h_mod - h_lab)
        model_err.append(h_rm - h_lab)
        lab_ref.append(h_lab)
    s678 = d["sec678"]
    order = np.argsort(-s678[:, 0])
    for c, j in enumerate(ALONG_J, 1):
        xs = -s678[order, 0]
        h_lab = 2e-3 * s678[order, c]
        h_mod = np.interp(xs, x, height[:, j + YSHIFT - 1])
        h_rm = np.interp(xs, x, href[:, j + YSHIFT - 1])
        lab_err.append(h_mod - h_lab)
        model_err.append(h_rm - h_lab)
        lab_ref.append(h_lab)
    e, em, lr = np.concatenate(lab_err), np.concatenate(model_err), np.concatenate(lab_ref)
    out["lab_points"] = int(lr.size)
    out["rel_rms_vs_lab"] = float(np.sqrt(np.mean(e ** 2)) / np.sqrt(np.mean(lr ** 2)))
    out["reference_model_rel_rms_vs_lab"] = float(np.sqrt(np.mean(em ** 2)) / np.sqrt(np.mean(lr ** 2)))
    return out
