"""Physical invariants of the scheme, which pin the restatement (and, in the
GPU variants, the kernels) independently of how either is written:

  lake at rest   still water over rough bathymetry with dry land stays
                 still, up to the limiter's guard: the well-balanced pressure
                 form 0.5 g (eta^2 + 2 eta h) (fluxes.F:1359-1373) and the
                 wet/dry face rules (bc.F:221-293) give zero fluxes, but the
                 van Leer limiter replaces a slope |t| <= SMALL = 1e-6 by
                 SMALL*sign(t) (fluxes.F:1602-1630), which puts ~0.5e-6 m
                 corrections on flat water; eta stays within 1e-5 m and u, v
                 within 1e-4 m/s (bounded: the same after 30 and 240 steps)
  volume         in a closed basin without wavemaker or sponge the sum of
                 eta changes only by rounding (the update is in flux form,
                 etauv_solver.F:88-110)
  mirror         a state and bathymetry symmetric in y stay symmetric, up to
                 the same guard: sign(+0) = +1 for the exactly zero slope at
                 the centre line, so symmetry holds to ~1e-6 m
  dispersion     the WK_REG wavenumber solves Nwogu's dispersion relation
                 with alpha = -0.39 (wavemaker.F:2378-2392)

The oracle runs on CPU; the GPU variants are marked gpu.
"""
import math

import numpy as np
import pytest

from helpers import G

GRAV = 9.81


def _basin(M, N, kind, seed=3):
    """(params, depth, eta0) of a walled basin with no wavemaker or sponge."""
    rng = np.random.default_rng(seed)
    x = (np.arange(M) + 0.5) / M
    y = (np.arange(N) + 0.5) / N
    X, Y = np.meshgrid(x, y, indexing="ij")
    p = {"Mglob": M, "Nglob": N, "DX": 1.0, "DY": 1.0, "PERIODIC": False, "WAVEMAKER": "NONE",
         "DISPERSION": True, "MinDepth": 0.01, "CFL": 0.5}
    if kind == "lake":
        # rough bottom and an island whose top is dry land
        depth = 2.0 + 0.3 * rng.standard_normal((M, N))
        island = 3.5 * np.exp(-(((X - 0.6) / 0.15) ** 2 + ((Y - 0.5) / 0.2) ** 2))
        depth = depth - island
        eta = np.where(depth > 0.0, 0.0, 0.0)
    elif kind == "volume":
        depth = 3.0 + 0.5 * np.sin(3.0 * X) * np.cos(2.0 * Y)
        eta = 0.05 * np.exp(-(((X - 0.4) / 0.1) ** 2 + ((Y - 0.45) / 0.12) ** 2))
    else:  # mirror: symmetric about the y centre line
        depth = 3.0 + 0.4 * np.cos(2.0 * math.pi * X) + 0.3 * (Y - 0.5) ** 2
        eta = 0.04 * np.exp(-(((X - 0.35) / 0.1) ** 2 + ((Y - 0.5) / 0.15) ** 2))
    return p, np.asfortranarray(depth), np.asfortranarray(eta)


def _oracle_run(oracle_mod, fw, p, depth, eta, nsteps):
    o = oracle_mod.Oracle(fw.with_defaults(p))
    o["Depth"][G:-G, G:-G] = depth
    o["Eta"][G:-G, G:-G] = eta
    o.init()
    for _ in range(nsteps):
        assert o.step() == 0
    return o


# the limiter guard bounds the departures (see the module docstring)
GUARD_TOL = 1e-5     # eta, m
GUARD_TOL_U = 1e-4   # u, v, m/s


def _check_lake(get, tol, tol_u):
    mask = get("MASK")[G:-G, G:-G] > 0
    eta = get("Eta")[G:-G, G:-G]
    assert mask.any() and not mask.all()  # there is dry land
    assert float(np.abs(eta[mask]).max()) <= tol
    assert float(np.abs(get("U")[G:-G, G:-G]).max()) <= tol_u
    assert float(np.abs(get("V")[G:-G, G:-G]).max()) <= tol_u


def test_lake_at_rest_oracle(oracle_mod, fw):
    p, depth, eta = _basin(40, 32, "lake")
    o = _oracle_run(oracle_mod, fw, p, depth, eta, 30)
    _check_lake(lambda n: o[n], GUARD_TOL, GUARD_TOL_U)


def test_volume_closed_basin_oracle(oracle_mod, fw):
    p, depth, eta = _basin(48, 40, "volume")
    o = _oracle_run(oracle_mod, fw, p, depth, eta, 40)
    v0 = float(eta.sum())
    v = float(o["Eta"][G:-G, G:-G].sum())
    assert abs(v - v0) <= 1e-12 * float(np.abs(eta).sum())
    assert float(np.abs(o["Eta"][G:-G, G:-G] - eta).max()) > 1e-3  # it did move


def test_mirror_symmetry_oracle(oracle_mod, fw):
    p, depth, eta = _basin(48, 40, "mirror")
    assert np.array_equal(depth, depth[:, ::-1])
    o = _oracle_run(oracle_mod, fw, p, depth, eta, 30)
    e = o["Eta"][G:-G, G:-G]
    assert float(np.abs(e).max()) > 1e-3
    assert float(np.abs(e - e[:, ::-1]).max()) <= GUARD_TOL
    u, v = o["U"][G:-G, G:-G], o["V"][G:-G, G:-G]
    assert float(np.abs(u - u[:, ::-1]).max()) <= GUARD_TOL_U
    assert float(np.abs(v + v[:, ::-1]).max()) <= GUARD_TOL_U


@pytest.mark.parametrize("T,h", [(6.0, 5.0), (10.0, 20.0), (4.0, 1.0)])
def test_wk_reg_wavenumber_solves_nwogu_relation(oracle_mod, fw, T, h):
    """omega^2 = g k^2 h (1 - (alpha + 1/3)(kh)^2) / (1 - alpha (kh)^2)."""
    theta = 30.0
    p = {"Mglob": 16, "Nglob": 16, "DX": 1.0, "DY": 1.0, "WAVEMAKER": "WK_REG", "AMP_WK": 0.1,
         "Tperiod": T, "DEP_WK": h, "Xc_WK": 5.0, "Theta_WK": theta, "Time_ramp": 1.0}
    o = oracle_mod.Oracle(fw.with_defaults(p))
    o["Depth"][...] = h
    o.init()
    pi_sp = float(np.float32(3.141592653))
    k = o.scalar("rlamda") / math.sin(theta * pi_sp / 180.0)
    # the literals -0.39 and 1./3. are default REAL in the reference
    alpha = float(np.float32(-0.39))
    third = float(np.float32(1.0 / 3.0))
    w = 2.0 * pi_sp / T
    kh = k * h
    lhs = w * w
    rhs = GRAV * k * k * h * (1.0 - (alpha + third) * kh * kh) / (1.0 - alpha * kh * kh)
    assert abs(lhs - rhs) <= 1e-12 * lhs
    # and the physical root: within 2 % of the exact linear wavenumber
    # (omega^2 = g k tanh(k h)), which Nwogu's relation approximates
    ke = w / math.sqrt(GRAV * h)
    for _ in range(60):
        f = GRAV * ke * math.tanh(ke * h) - w * w
        df = GRAV * math.tanh(ke * h) + GRAV * ke * h / math.cosh(ke * h) ** 2
        ke -= f / df
    assert abs(k - ke) <= 0.02 * ke


# --------------------------------------------------------------------------
# GPU: the same invariants through the C ABI, FP64 and mixed precision
# --------------------------------------------------------------------------
def _gpu_run(fw, p, depth, eta, nsteps, precision):
    s = fw.Solver(fw.with_defaults(p), precision=precision)
    s.init(depth, eta=eta)
    st = s.step(nsteps)
    assert st == 0
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("FP64", GUARD_TOL), ("MIXED", GUARD_TOL)])
def test_lake_at_rest_gpu(fw, precision, tol):
    p, depth, eta = _basin(40, 32, "lake")
    s = _gpu_run(fw, p, depth, eta, 30, precision)
    _check_lake(s.get, tol, GUARD_TOL_U)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("FP64", 1e-12), ("MIXED", 2e-6)])
def test_volume_closed_basin_gpu(fw, precision, tol):
    p, depth, eta = _basin(48, 40, "volume")
    s = _gpu_run(fw, p, depth, eta, 40, precision)
    v0 = float(eta.sum())
    e = s.get("Eta")[G:-G, G:-G]
    assert abs(float(e.sum()) - v0) <= tol * float(np.abs(eta).sum())
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("FP64", GUARD_TOL), ("MIXED", 2 * GUARD_TOL)])
def test_mirror_symmetry_gpu(fw, precision, tol):
    p, depth, eta = _basin(48, 40, "mirror")
    s = _gpu_run(fw, p, depth, eta, 30, precision)
    e = s.get("Eta")[G:-G, G:-G]
    assert float(np.abs(e - e[:, ::-1]).max()) <= tol
    s.close()
