"""Whole FP64 runs against the oracle on the benchmark configurations
themselves, not only on small parity cases.

* The 250 x 500 planar beach at full size (1:20 slope to dry land, seeded
  smoothed bathymetry noise, WK_REG H = 0.3 m, T = 6 s, periodic in y,
  west sponge, dispersion and breaking on): 300 whole steps, compared every
  50 steps.
* Two 256 x 256 crops of the 2048^2 shoal configuration (dx = 2 m): the west
  corner with the JON_2D wavemaker (50 frequencies x 30 directions, cos^2s
  spreading, seeded phases) and the sponge, and the shoreline strip with its
  dry land, both from a seeded random state so that the first steps already
  move water: 50 whole steps each.

Tolerance: eta, u, v within 1e-9 of their scale over the interior; MASK
bit-exact.  The FP64 kernels keep the reference's operation order, so the
two differ only where CUDA's libm rounds exp/sin/cos/tanh/atan2 in another
last bit than glibc, and those differences stay far below 1e-9.
"""
import numpy as np
import pytest

from helpers import interior, make_pair, maxrel

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _run_and_compare(s, o, nsteps, every):
    done = 0
    while done < nsteps:
        k = min(every, nsteps - done)
        s.step(k)
        for _ in range(k):
            o.step()
        done += k
        assert np.array_equal(s.get("MASK"), o["MASK"]), "MASK after %d steps" % done
        for name in ("Eta", "U", "V"):
            e = maxrel(interior(s.get(name)), interior(o[name]))
            assert e <= TOL, "%s after %d steps: %.3e" % (name, done, e)
    t_gpu, t_ref = s.scalar("TIME"), o.scalar("TIME")
    assert abs(t_gpu - t_ref) <= 1e-12 * t_ref, (t_gpu, t_ref)
    return t_ref


def test_planar_beach_full_size_300_steps(fw, oracle_mod):
    p, depth, _ = fw.cases.planar_beach()          # 250 x 500, the configuration as stated
    assert (p["Mglob"], p["Nglob"]) == (250, 500)
    s, o = make_pair(fw, oracle_mod, p, depth)
    t = _run_and_compare(s, o, 300, 50)
    assert t > 10.0                                 # ~14 s of model time: waves on the slope
    # waves from the wavemaker fill the flat part (x < 100 m)
    assert float(np.abs(interior(s.get("Eta"))[:100]).max()) > 0.05
    s.close()
    o.close()


def _crop(fw, i0, j0, n=256, seed=5, wavemaker=True):
    p, depth, phases = fw.cases.shoal_jonswap(seed=seed)
    depth = np.asfortranarray(depth[i0:i0 + n, j0:j0 + n])
    p.update({"Mglob": n, "Nglob": n})
    if not wavemaker:
        p["WAVEMAKER"] = "NONE"
        phases = None
    state = fw.cases.random_state(n, n, seed=seed + 1, eta_amp=0.3, u_amp=0.4, smooth=4.0)
    eta = state[0]
    # dry cells keep the state the initialisation gives them
    wet = depth > 0.05
    state = (np.where(wet, eta, 0.0), np.where(wet, state[1], 0.0), np.where(wet, state[2], 0.0))
    return p, depth, state, phases


@pytest.mark.parametrize("where", ["wavemaker_corner", "shoreline"])
def test_shoal_crop_50_steps(fw, oracle_mod, where):
    if where == "wavemaker_corner":
        p, depth, state, phases = _crop(fw, 0, 896)
        assert p["WAVEMAKER"] == "JON_2D" and p["Nfreq"] == 50 and p["Ntheta"] == 30
    else:
        # cells 1792..2047 in x: the 1:50 slope through the shoreline
        # (x = 3896 m, cell 1948) and 200 m of land behind it
        p, depth, state, phases = _crop(fw, 1792, 896, wavemaker=False)
        assert (depth < 0).any() and (depth > 0).any()
    s, o = make_pair(fw, oracle_mod, p, depth, state, phases)
    _run_and_compare(s, o, 50, 25)
    s.close()
    o.close()


def test_shoal_full_size_3_steps(fw, oracle_mod):
    """The 2048 x 2048 shoal workload itself (JON_2D 50 x 30 cos^2s from
    rest, seed of the benchmark): three whole FP64 steps against the oracle
    at full size (the oracle takes about 5 s a step on 16 cores)."""
    p, depth, phases = fw.cases.shoal_jonswap(seed=2024)
    assert (p["Mglob"], p["Nglob"]) == (2048, 2048)
    s, o = make_pair(fw, oracle_mod, p, depth, None, phases)
    _run_and_compare(s, o, 3, 3)
    s.close()
    o.close()

