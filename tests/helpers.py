"""Shared set-up of matching (GPU solver, CPU oracle) pairs for the tests."""
import numpy as np

G = 3  # ghost cells


def interior(a):
    return a[G:-G, G:-G]


def make_pair(fw, oracle_mod, params, depth, state=None, phases=None, precision="FP64"):
    p = fw.with_defaults(params)
    s = fw.Solver(p, precision=precision)
    eta = u = v = None
    if state is not None:
        eta, u, v = state
    s.init(depth, eta, u, v, phases)
    o = oracle_mod.Oracle(p)
    o["Depth"][G:-G, G:-G] = depth
    if state is not None:
        o["Eta"][G:-G, G:-G] = eta
        o["U"][G:-G, G:-G] = u
        o["V"][G:-G, G:-G] = v
    if phases is not None:
        o.set_phases(phases)
    o.init()
    return s, o


def maxrel(a, b, floor=1e-6):
    scale = max(float(np.abs(b).max()), floor)
    return float(np.abs(a - b).max()) / scale


def sloped_beach(Mglob, Nglob, h0=1.5, h1=-1.0, seed=0, noise=0.01):
    """A linear beach from h0 (x = 0) to h1 (x = end) with smooth noise:
    it has a shoreline, dry land and a wet/dry front."""
    x = np.linspace(0.0, 1.0, Mglob)
    d = np.repeat((h0 + (h1 - h0) * x)[:, None], Nglob, axis=1)
    rng = np.random.default_rng(seed)
    d = d + noise * rng.standard_normal((Mglob, Nglob))
    return np.asfortranarray(d)
