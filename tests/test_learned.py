"""The learned coarse-grid correction (a spec extension without a
reference counterpart).

CPU: the numpy reference of the network (oracle/fw_net_oracle.py) against
finite differences, in float64.
GPU: the library's forward pass and every parameter gradient against that
reference (with BF16 rounding of weights and activations as the GPU stores
them), and the effect of training on held-out one-step errors.
"""
import numpy as np
import pytest


def _rand_params(ref, seed):
    rng = np.random.default_rng(seed)
    p = []
    for ci, co, _ in ref.LAYERS:
        cin_real = 5 if ci == 8 else ci
        w = rng.normal(0.0, np.sqrt(2.0 / (9 * cin_real)), size=(9, ci, co))
        w[:, cin_real:, :] = 0.0
        p.append(w.ravel())
        p.append(rng.normal(0.0, 0.1, size=co))
    return np.concatenate(p).astype(np.float32)


def test_reference_gradients_by_finite_differences():
    import fw_net_oracle as ref
    rng = np.random.default_rng(1)
    params = _rand_params(ref, 2).astype(np.float64)
    x = rng.normal(size=(2, 5, 6, 5))
    t = rng.normal(size=(2, 5, 6, 3))
    w = (rng.uniform(size=(2, 5, 6)) > 0.3).astype(float)
    loss, g = ref.loss_grad(params, x, t, w, bf16=False)
    eps = 1e-6
    for k in rng.choice(params.size, size=40, replace=False):
        if k < 9 * 8 * 32 and (k // 32) % 8 >= 5:
            continue  # padding input channels
        pp, pm = params.copy(), params.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (ref.loss_grad(pp, x, t, w, bf16=False)[0] - ref.loss_grad(pm, x, t, w, bf16=False)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def _check_forward(y, y_ref):
    """The tensor cores add in another order than the reference, so a hidden
    activation now and then rounds to the neighbouring BF16 value; the
    three layers after it spread that 0.4 % step over a 7 x 7 patch of
    outputs.  Most outputs agree to float rounding, a few by such a step."""
    e = np.abs(y - y_ref)
    scale = float(np.abs(y_ref).max())
    assert float(e.max()) <= 1e-2 * scale
    assert float(np.quantile(e, 0.9)) <= 1e-5 * scale


@pytest.mark.gpu
def test_gpu_forward_and_gradients_match_reference(fw):
    import torch
    import fw_net_oracle as ref
    net = fw.learned.Net(seed=3)
    assert net.n == ref.num_params()
    params = _rand_params(ref, 4)
    net.set_params(params)
    rng = np.random.default_rng(5)
    x = rng.normal(size=(2, 9, 13, 5)).astype(np.float32)
    t = rng.normal(size=(2, 9, 13, 3)).astype(np.float32)
    w = (rng.uniform(size=(2, 9, 13)) > 0.2).astype(np.float32)
    dev = torch.device("cuda")
    X, T, Wm = (torch.from_numpy(a).to(dev).contiguous() for a in (x, t, w))
    y = net.forward(X).cpu().numpy()
    y_ref, _ = ref.forward(params, x, bf16=True)
    _check_forward(y, y_ref)
    loss = net.loss_grad(X, T, Wm)
    loss_ref, g_ref = ref.loss_grad(params, x, t, w, bf16=True)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    g = net.grads()
    off = 0
    for ci, co, _ in ref.LAYERS:
        n = 9 * ci * co + co
        a, b = g[off:off + n], g_ref[off:off + n]
        assert np.linalg.norm(a - b) <= 2e-3 * np.linalg.norm(b), (ci, co, np.linalg.norm(a - b) / np.linalg.norm(b))
        off += n
    net.close()


@pytest.mark.gpu
def test_gpu_forward_and_gradients_several_tiles(fw):
    """Images wider than one 128-pixel tile, with a row count that is not a
    multiple of the tensor-core kernel's four rows, two to a batch: the
    tiles' halos, the zero fill at every edge and the partial last tiles."""
    import torch
    import fw_net_oracle as ref
    net = fw.learned.Net(seed=3)
    params = _rand_params(ref, 6)
    net.set_params(params)
    rng = np.random.default_rng(7)
    x = rng.normal(size=(2, 11, 150, 5)).astype(np.float32)
    t = rng.normal(size=(2, 11, 150, 3)).astype(np.float32)
    w = (rng.uniform(size=(2, 11, 150)) > 0.2).astype(np.float32)
    dev = torch.device("cuda")
    X, T, Wm = (torch.from_numpy(a).to(dev).contiguous() for a in (x, t, w))
    y = net.forward(X).cpu().numpy()
    y_ref, _ = ref.forward(params, x, bf16=True)
    _check_forward(y, y_ref)
    loss = net.loss_grad(X, T, Wm)
    loss_ref, g_ref = ref.loss_grad(params, x, t, w, bf16=True)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    g = net.grads()
    off = 0
    for ci, co, _ in ref.LAYERS:
        n = 9 * ci * co + co
        a, b = g[off:off + n], g_ref[off:off + n]
        assert np.linalg.norm(a - b) <= 2e-3 * np.linalg.norm(b), (ci, co, np.linalg.norm(a - b) / np.linalg.norm(b))
        off += n
    net.close()


@pytest.mark.gpu
def test_correct_run_equals_step_and_correct(fw):
    """fw_correct_run (graph replays of two step + correction pairs, and an
    odd last pair) computes what stepping and correcting one by one does."""
    case = _barred_case(fw, 5)
    pc, dc = fw.learned.coarse_case(fw.with_defaults(case[0]), case[1])
    net = fw.learned.Net(seed=7)
    runs = []
    for mode in ("loop", "graph"):
        s = fw.Solver(fw.with_defaults(pc), precision="MIXED")
        s.init(dc, phases=case[2])
        if mode == "loop":
            for _ in range(7):
                s.step(1)
                net.correct(s, wait=False)
            s.sync()
        else:
            assert net.correct_run(s, 7) == 0
        runs.append({n: s.get(n) for n in ("Eta", "U", "V", "Ubar", "Vbar", "MASK")})
        s.close()
    for name in runs[0]:
        assert np.array_equal(runs[0][name], runs[1][name]), name
    assert np.abs(runs[0]["Eta"]).max() > 0
    net.close()


def _barred_case(fw, seed, M=256, N=128):
    p, d, ph, _ = fw.cases.barred_beach(M, N, 1.0, seed=seed, wk_from_shore=150.0, nfreq=16, ntheta=4,
                                        shore_from_east=40.0, Hmo=0.8, Sponge_west_width=30.0)
    p["DT_fixed"] = 0.04
    return (p, d, ph)


@pytest.mark.gpu
def test_training_reduces_held_out_error(fw):
    """Pairs from three seeded barred beaches (fine dx = 1 m, coarse 2 m, the
    solver generating both), 600 Adam steps, then on a fourth, held-out
    beach: the one-step coarse error with the correction is at least 30 %
    below the plain coarse step's, and a 200-step corrected coarse run is
    no further from the restricted fine run in eta than the plain one."""
    L = fw.learned
    X, T, W = [], [], []
    for seed in (1, 2, 3):
        x, t, w = L.make_pairs(_barred_case(fw, seed), 200, every=2)
        X.append(x)
        T.append(t)
        W.append(w)
    X, T, W = np.concatenate(X), np.concatenate(T), np.concatenate(W)
    assert np.sqrt((T ** 2).mean()) > 1e-3  # the coarse step does err
    held = _barred_case(fw, 9)
    xh, th, wh = L.make_pairs(held, 200, every=2)
    net = L.Net(seed=0)
    losses = L.train(net, X, T, W, iters=600, batch=8, lr=2e-3)
    assert np.mean(losses[-50:]) < 0.5 * np.mean(losses[:20])
    e_plain, e_net = L.one_step_error(net, xh, th, wh)
    assert e_net <= 0.7 * e_plain, (e_net, e_plain)
    fine = L.fine_run(held, 400)
    plain, _ = L.rollout(held, 200)
    corr, applied = L.rollout(held, 200, net=net)
    assert applied == 200
    f = L.restrict(fine["Eta"])
    m = (plain["MASK"] > 0) & (corr["MASK"] > 0)
    r_plain = np.sqrt(np.mean((plain["Eta"] - f)[m] ** 2))
    r_corr = np.sqrt(np.mean((corr["Eta"] - f)[m] ** 2))
    assert r_corr <= r_plain, (r_corr, r_plain)
    # the eta correction is projected to zero mean over wet cells: the
    # corrected run keeps the plain run's volume budget
    net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_correction_fallback_checks(fw, precision):
    """fw_correct keeps the plain step when a check fails: a correction above
    max_corr, a volume drift (the raw eta correction's mean, which the
    projection would remove) above half of max_corr, or a wet cell pushed to
    or below MinDepth; fw_net_last_check reports the checked values.  A
    correction acts only on cells whose 3 x 3 neighbourhood is wet (5 x 5
    with fw_net_set_shore_band(2), every wet cell with 0).
    The output layer's weights are zero here, so the correction is its bias:
    eta bias b_e and u bias b_u, in metres and m/s."""
    import fw_net_oracle as ref
    params, depth, _ = fw.cases.planar_beach(Mglob=64, Nglob=40, seed=2)
    depth = np.array(depth)
    depth[10:14, 5:9] = 0.03          # a patch of shallow wet cells (MinDepth 0.01 m)
    depth[52:, 28:] = -0.5            # an island: land and a shoreline
    p = fw.with_defaults(params)
    net = fw.learned.Net(seed=3)
    base = net.params()
    co = ref.LAYERS[-1][1]
    nlast = 9 * ref.LAYERS[-1][0] * co + co

    def run(b_e, b_u, max_corr, shallow=True, band=1):
        d = depth if shallow else np.maximum(depth, np.where(depth > 0, 0.2, depth))
        s = fw.Solver(p, precision=precision)
        s.init(d)
        s.step(2)
        w = base.copy()
        w[-nlast:] = 0.0
        w[-co:][0] = b_e * fw.learned.OUT_SCALE
        w[-co:][1] = b_u * fw.learned.OUT_SCALE
        net.set_params(w)
        eta0, u0 = s.get("Eta"), s.get("U")
        net.set_shore_band(band)
        applied = net.correct(s, max_corr=max_corr)
        eta1, u1 = s.get("Eta"), s.get("U")
        m = s.get("MASK") > 0
        k = band
        wet9 = np.zeros_like(m)
        wet9[k:m.shape[0] - k, k:m.shape[1] - k] = np.all(
            [m[k + a:m.shape[0] - k + a, k + b:m.shape[1] - k + b] for a in range(-k, k + 1) for b in range(-k, k + 1)],
            axis=0)
        s.close()
        return applied, eta0, eta1, u0, u1, wet9, net.last_check()

    # size cap
    a, e0, e1, u0, u1, _, c = run(0.0, 0.3, 0.2)
    assert not a and np.array_equal(e0, e1) and np.array_equal(u0, u1)
    assert not c["applied"] and abs(c["max_abs"] - 0.3) < 1e-6 and c["dry_m"] == 0.0
    # volume drift: a uniform rise of 0.15 m against max_corr 0.2 m
    a, e0, e1, u0, u1, _, c = run(0.15, 0.0, 0.2)
    assert not a and np.array_equal(e0, e1) and np.array_equal(u0, u1)
    assert abs(c["mean_eta"] - 0.15) < 1e-6
    # a uniform fall of 0.04 m would dry the 0.03 m patch
    a, e0, e1, u0, u1, _, c = run(-0.04, 0.05, 0.2)
    assert not a and np.array_equal(e0, e1) and np.array_equal(u0, u1)
    assert abs(c["dry_m"] - 0.02) < 1e-3
    # the same without shallow cells passes: the uniform eta part is
    # projected away (volume kept) and u gets its 0.05 m/s on the cells
    # whose neighbourhood is wet, nothing at the shoreline; with a band of 2
    # cells the 5 x 5 neighbourhood, with 0 every wet cell
    for band in (1, 2, 0):
        a, e0, e1, u0, u1, wet9, c = run(-0.04, 0.05, 0.2, shallow=False, band=band)
        assert a and c["applied"] and c["cells"] == float(wet9[3:-3, 3:-3].sum())
        assert float(np.abs(e1 - e0).max()) <= 1e-6
        du = (u1 - u0)[3:-3, 3:-3]
        m9 = wet9[3:-3, 3:-3]
        assert m9.any() and (~m9).any()
        assert np.allclose(du[m9], 0.05, rtol=0, atol=1e-6)
        assert np.array_equal(du[~m9], np.zeros_like(du[~m9]))
    with pytest.raises(fw.FwError):
        net.set_shore_band(4)
    net.close()
