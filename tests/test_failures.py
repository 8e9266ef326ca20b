"""Failure reporting: CHECK_BLOWUP (misc.F:394-433) and the NaN check of
CHECK_STATISTICS (statistics.F:192-210) as step statuses, and the bounded
device waits of the TMA-staged flux tiles and of the tensor-core
convolutions.

Every failure here is made on the host: eta above EtaBlowVal or a NaN
written into the state through fw_set_field, and wait limits lowered to one
poll so that the kernels' bounded waits run out.  Nothing faults, traps or
hangs the GPU: an expired wait makes its kernel give up, wait for its own
copies (and MMAs) with the full limit and return.  Each test then uses the
same context or network again and checks that it works.
"""
import numpy as np
import pytest

from helpers import G

pytestmark = pytest.mark.gpu

FW_ERR_BLOWUP, FW_ERR_NAN, FW_ERR_TIMEOUT = -4, -5, -10


def _case(fw, precision, tma=False):
    params, depth, _ = fw.cases.planar_beach(Mglob=64, Nglob=40, seed=2)
    p = fw.with_defaults(params)
    eta, u, v = fw.cases.random_state(64, 40, seed=3)
    s = fw.Solver(p, precision=precision)
    s.init(depth, eta, u, v)
    if tma:
        t = s.tuning()
        t.update({"flux_x": 8, "flux_y": 16, "flux_x_tma": 1, "flux_y_tma": 1})
        s.set_tuning(t)
    return s, depth, (eta, u, v)


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
@pytest.mark.parametrize("nsteps", [1, 3])
def test_blowup_reported(fw, precision, nsteps):
    s, depth, state = _case(fw, precision)
    assert s.step(2, check=False) == 0
    s.set_scalar("EtaBlowVal", 2.0)
    eta = s.get("Eta")
    # a 7 x 7 patch 3 m high in 5 m of water, 20 m from the west edge
    eta[G + 17:G + 24, G + 15:G + 22] = 3.0
    s.set("Eta", eta)
    assert s.step(nsteps, check=False) == FW_ERR_BLOWUP
    with pytest.raises(fw.FwError) as e:
        s.set("Eta", eta)
        s.step(1)
    assert e.value.status == FW_ERR_BLOWUP
    # the context is still usable: a clean state steps without a status
    s.set_scalar("EtaBlowVal", 100.0)
    s.init(depth, *state)
    assert s.step(nsteps, check=False) == 0
    assert np.isfinite(s.get("Eta")).all()
    s.close()


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_nan_reported(fw, precision):
    s, depth, state = _case(fw, precision)
    assert s.step(1, check=False) == 0
    eta = s.get("Eta")
    eta[G + 20, G + 10] = np.nan
    s.set("Eta", eta)
    assert s.step(1, check=False) == FW_ERR_NAN
    # NaN stays NaN in later steps too (CHECK_BLOWUP sees it as +inf)
    assert s.step(2, check=False) == FW_ERR_NAN
    s.init(depth, *state)
    assert s.step(2, check=False) == 0
    s.close()


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_flux_tile_wait_expiry_reported(fw, precision):
    """WAIT_LIMIT = 1 poll: the TMA-staged flux tiles give up before their
    copies land, write NaN fluxes, drain the copies and return; the step
    reports FW_ERR_NAN.  With the default limit back, the same context runs
    two steps bit for bit like a fresh one."""
    s, depth, state = _case(fw, precision, tma=True)
    assert s.scalar("WAIT_LIMIT") == 0.0
    s.set_scalar("WAIT_LIMIT", 1)
    assert s.scalar("WAIT_LIMIT") == 1.0
    assert s.step(1, check=False) == FW_ERR_NAN
    s.set_scalar("WAIT_LIMIT", 0)
    s.init(depth, *state)
    assert s.step(2, check=False) == 0
    got = s.get("Eta")
    s.close()
    ref, _, _ = _case(fw, precision, tma=True)
    assert ref.step(2, check=False) == 0
    assert np.array_equal(got, ref.get("Eta"))
    ref.close()


def test_conv_wait_expiry_reported(fw):
    """The tensor-core convolutions with a one-poll wait limit: the kernels
    give up, drain their loads and MMAs, free TMEM and return;
    fw_net_loss_grad reports FW_ERR_TIMEOUT and clears the status.  With the
    default limit back, the same network gives the loss and gradients of a
    fresh network with the same weights (the loss to its summation order)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)
    B, H, W = 2, 12, 300   # three 128-pixel tiles across, partial row tiles
    x = torch.from_numpy(rng.normal(size=(B, H, W, 5)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.normal(size=(B, H, W, 3)).astype(np.float32)).cuda()
    m = torch.ones((B, H, W), dtype=torch.float32, device="cuda")
    net = fw.learned.Net(seed=4)
    net.set_wait_limit(1)
    with pytest.raises(fw.FwError) as e:
        net.loss_grad(x, t, m)
    assert e.value.status == FW_ERR_TIMEOUT
    net.set_wait_limit(0)
    loss = net.loss_grad(x, t, m)
    g = net.grads()
    ref = fw.learned.Net(seed=4)
    loss_ref = ref.loss_grad(x, t, m)
    # the loss is summed with atomics (order varies); the gradients are not
    assert np.isfinite(loss) and abs(loss - loss_ref) <= 1e-12 * abs(loss_ref)
    assert np.array_equal(g, ref.grads())
    net.close()
    ref.close()
