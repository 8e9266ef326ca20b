"""The learned coarse-grid correction (spec extension; no reference
counterpart): a small convolutional network that corrects each step of a
2x-coarser run toward the fine-grid solution.

  Net             ctypes handle of the library's network (fw_net_*): forward,
                  loss + gradients, Adam, parameters
  restrict        2x2 cell averages of a fine field (coarse cell I takes
                  the fine cells 2I-1, 2I)
  make_pairs      one-step training pairs generated by the solver itself:
                  the coarse state restricted from a fine run at time t, and
                  the difference between the restricted fine state at the
                  next coarse time and one plain coarse step from it
  train           Adam on the pairs (the network's own forward and backward
                  kernels on the GPU)
  rollout         a coarse run with fw_correct after every step

Inputs are (eta, u, v, depth / FW_NET_DEPTH_SCALE, MASK) of the coarse
interior, outputs FW_NET_OUT_SCALE times the corrections of (eta, u, v).
The coarse run uses twice the fine run's fixed time step (DT_fixed).
"""
import ctypes

import numpy as np

from .params import with_defaults
from .solver import FwError, Solver, load_library

DEPTH_SCALE = 10.0
OUT_SCALE = 100.0
G = 3


def _bind(L):
    vp, ip, fp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.fw_net_create.argtypes = [ctypes.c_ulonglong, ctypes.POINTER(vp)]
    L.fw_net_destroy.argtypes = [vp]
    L.fw_net_num_params.argtypes = [vp]
    L.fw_net_num_params.restype = ctypes.c_longlong
    L.fw_net_get_params.argtypes = [vp, vp]
    L.fw_net_set_params.argtypes = [vp, vp]
    L.fw_net_get_grads.argtypes = [vp, vp]
    L.fw_net_forward.argtypes = [vp, vp, ip, ip, ip, vp, vp]
    L.fw_net_loss_grad.argtypes = [vp, vp, vp, vp, ip, ip, ip, ctypes.POINTER(ctypes.c_double), vp]
    L.fw_net_adam.argtypes = [vp, fp, fp, fp, fp, vp]
    L.fw_net_set_wait_limit.argtypes = [vp, ctypes.c_uint]
    L.fw_correct.argtypes = [vp, vp, ctypes.c_double, ctypes.POINTER(ip)]
    L.fw_correct_run.argtypes = [vp, vp, ip, ctypes.c_double, ctypes.POINTER(ip)]
    L.fw_net_last_check.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.fw_net_set_shore_band.argtypes = [vp, ip]
    return L


class Net:
    """The library's network; tensors are torch CUDA float32, channels-last."""

    def __init__(self, seed=0):
        self.L = _bind(load_library())
        h = ctypes.c_void_p()
        rc = self.L.fw_net_create(int(seed), ctypes.byref(h))
        if rc != 0:
            raise FwError(rc, "fw_net_create")
        self.h = h
        self.n = int(self.L.fw_net_num_params(h))

    def close(self):
        if getattr(self, "h", None):
            self.L.fw_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        a = np.zeros(self.n, dtype=np.float32)
        self._ck(self.L.fw_net_get_params(self.h, a.ctypes.data), "get_params")
        return a

    def set_params(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        assert a.size == self.n
        self._ck(self.L.fw_net_set_params(self.h, a.ctypes.data), "set_params")

    def grads(self):
        a = np.zeros(self.n, dtype=np.float32)
        self._ck(self.L.fw_net_get_grads(self.h, a.ctypes.data), "get_grads")
        return a

    def forward(self, x):
        import torch
        B, H, W, C = x.shape
        assert C == 5 and x.is_cuda and x.dtype == torch.float32 and x.is_contiguous()
        y = torch.empty((B, H, W, 3), dtype=torch.float32, device=x.device)
        s = torch.cuda.current_stream().cuda_stream
        self._ck(self.L.fw_net_forward(self.h, x.data_ptr(), B, H, W, y.data_ptr(), s), "forward")
        return y

    def loss_grad(self, x, target, wmask):
        import torch
        B, H, W, _ = x.shape
        loss = ctypes.c_double()
        s = torch.cuda.current_stream().cuda_stream
        self._ck(self.L.fw_net_loss_grad(self.h, x.data_ptr(), target.data_ptr(), wmask.data_ptr(), B, H, W,
                                         ctypes.byref(loss), s), "loss_grad")
        return loss.value

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        import torch
        s = torch.cuda.current_stream().cuda_stream
        self._ck(self.L.fw_net_adam(self.h, float(lr), float(beta1), float(beta2), float(eps), s), "adam")

    def set_wait_limit(self, polls=0):
        """Polls of the tensor-core kernels' bounded waits (0 = default)."""
        self._ck(self.L.fw_net_set_wait_limit(self.h, int(polls)), "set_wait_limit")

    def correct(self, solver, max_corr=0.2, wait=True):
        """fw_correct on the solver's current state; with wait, whether the
        correction was applied (else the call only enqueues it)."""
        if not wait:
            self._ck(self.L.fw_correct(solver.ctx, self.h, float(max_corr), None), "fw_correct")
            return None
        ap = ctypes.c_int()
        self._ck(self.L.fw_correct(solver.ctx, self.h, float(max_corr), ctypes.byref(ap)), "fw_correct")
        return bool(ap.value)

    def set_shore_band(self, cells=1):
        """fw_net_set_shore_band: correct only where the (2 cells + 1)^2
        neighbourhood is wet (0: every wet cell)."""
        self._ck(self.L.fw_net_set_shore_band(self.h, int(cells)), "fw_net_set_shore_band")

    def last_check(self):
        """The checks of the last correct() that waited (fw_net_last_check):
        mean raw eta correction, cells corrected, max |correction|, MinDepth
        violation, applied."""
        out = (ctypes.c_double * 5)()
        self._ck(self.L.fw_net_last_check(self.h, out), "fw_net_last_check")
        return {"mean_eta": out[0], "cells": out[1], "max_abs": out[2], "dry_m": out[3], "applied": out[4] == 1.0}

    def correct_run(self, solver, nsteps, max_corr=0.2):
        """nsteps of (step + correction) on the solver through fw_correct_run:
        one graph replay per two pairs; returns the CHECK_BLOWUP status."""
        st = ctypes.c_int()
        self._ck(self.L.fw_correct_run(solver.ctx, self.h, int(nsteps), float(max_corr), ctypes.byref(st)),
                 "fw_correct_run")
        return st.value

    def _ck(self, rc, what):
        if rc != 0:
            raise FwError(rc, what)


def restrict(a):
    """2x2 cell average of an interior field (Mf x Nf -> Mf/2 x Nf/2)."""
    return 0.25 * (a[0::2, 0::2] + a[1::2, 0::2] + a[0::2, 1::2] + a[1::2, 1::2])


def coarse_case(params, depth):
    """The coarse twin of a fine case: DX, DY doubled, grid halved, depth
    restricted, DT_fixed doubled."""
    p = dict(params)
    p["Mglob"] //= 2
    p["Nglob"] //= 2
    p["DX"] = 2.0 * p["DX"]
    p["DY"] = 2.0 * p["DY"]
    p["DT_fixed"] = 2.0 * p["DT_fixed"]
    return p, np.asfortranarray(restrict(depth))


def features(eta, u, v, depth, mask):
    """[H=N][W=M][5] channels-last network input from interior (M, N) fields."""
    f = np.stack([eta, u, v, depth / DEPTH_SCALE, (mask > 0).astype(float)], axis=-1)
    return np.ascontiguousarray(f.transpose(1, 0, 2), dtype=np.float32)


def _interior(a):
    return a[G:-G, G:-G]


def _set_state(cs, eta, u, v, ubar, vbar, depth_c, mask):
    """Put a restricted state on the coarse solver (interior; ghosts by EXCHANGE)."""
    M, N = eta.shape
    full = {}
    for name, val in (("Eta", eta), ("U", u), ("V", v), ("Ubar", ubar), ("Vbar", vbar)):
        a = cs.get(name)
        a[G:-G, G:-G] = val
        full[name] = a
    H = full["Eta"] + cs.get("Depth")
    full["H"] = H
    full["HU"] = np.maximum(H, 0.0) * full["U"]
    full["HV"] = np.maximum(H, 0.0) * full["V"]
    for name, a in full.items():
        cs.set(name, a)
    m = cs.get("MASK")
    m[G:-G, G:-G] = mask
    cs.set("MASK", m)
    cs.exchange()


def make_pairs(case, nsteps_c, precision="MIXED", every=1, unroll=1, nudge=None):
    """Training pairs from one fine run of case = (params, depth, phases)
    (params with DT_fixed): returns (x [K, N, M, 5], target [K, N, M, 3],
    wmask [K, N, M]) as numpy float32, the target already multiplied by
    OUT_SCALE.

    Every `every` coarse steps the coarse twin starts from the restricted
    fine state and then runs on its own for `unroll` steps; each of those
    steps gives a pair: its input state (the restricted fine state first,
    then states the coarse solver evolved itself, as in a corrected run) and
    the difference between the restricted fine state one coarse step later
    and the coarse step's result.

    nudge = beta (0 < beta <= 1) instead: one coarse run over the whole
    trajectory that, after each step, moves beta of the way to the restricted
    fine state (eta, u, v, ubar, vbar): the state a run corrected by a
    network that removes a fraction beta of each step's error would be in.
    Every step gives a pair (every `every`-th is kept)."""
    pf, depth, phases = case
    pf = with_defaults(pf)
    pc, depth_c = coarse_case(pf, depth)
    fs = Solver(pf, precision=precision)
    fs.init(depth, phases=phases)
    cs = Solver(with_defaults(pc), precision=precision)
    cs.init(depth_c, phases=phases)
    xs, ts, ws = [], [], []

    def fine_state():
        return {n: restrict(_interior(fs.get(n))) for n in ("Eta", "U", "V", "Ubar", "Vbar")}

    # the restricted fine run at every coarse step (two fine steps each)
    ref, times = [fine_state()], [fs.scalar("TIME")]
    for _ in range(nsteps_c):
        fs.step(2)
        ref.append(fine_state())
        times.append(fs.scalar("TIME"))
    fs.close()
    dc = _interior(cs.get("Depth"))
    if nudge is not None:
        st = ref[0]
        mask = ((st["Eta"] + dc) > 1e-3).astype(np.int32)
        _set_state(cs, st["Eta"], st["U"], st["V"], st["Ubar"], st["Vbar"], dc, mask)
        cs.set_scalar("TIME", times[0])
        cur_in = {k: st[k] for k in ("Eta", "U", "V", "Ubar", "Vbar")}
        for k in range(nsteps_c):
            cs.step(1)
            c1 = {n: _interior(cs.get(n)) for n in ("Eta", "U", "V", "Ubar", "Vbar")}
            mc = _interior(cs.get("MASK"))
            cur = ref[k + 1]
            if k % every == 0:
                wet = ((mask > 0) & (mc > 0)).astype(np.float32)
                xs.append(features(cur_in["Eta"], cur_in["U"], cur_in["V"], dc, mask))
                tgt = np.stack([cur["Eta"] - c1["Eta"], cur["U"] - c1["U"], cur["V"] - c1["V"]], axis=-1) * OUT_SCALE
                ts.append(np.ascontiguousarray((tgt * wet[..., None]).transpose(1, 0, 2), dtype=np.float32))
                ws.append(np.ascontiguousarray(wet.T))
            nxt = {n: c1[n] + nudge * (cur[n] - c1[n]) for n in c1}
            mask = ((nxt["Eta"] + dc) > 1e-3).astype(np.int32)
            _set_state(cs, nxt["Eta"], nxt["U"], nxt["V"], nxt["Ubar"], nxt["Vbar"], dc, mask)
            cur_in = nxt
        cs.close()
        return np.stack(xs), np.stack(ts), np.stack(ws)
    for start in range(0, nsteps_c - unroll + 1, every):
        st = ref[start]
        mask = ((st["Eta"] + dc) > 1e-3).astype(np.int32)
        _set_state(cs, st["Eta"], st["U"], st["V"], st["Ubar"], st["Vbar"], dc, mask)
        cs.set_scalar("TIME", times[start])
        e_in, u_in, v_in = st["Eta"], st["U"], st["V"]
        for k in range(unroll):
            cs.step(1)
            ec, uc, vc = (_interior(cs.get(n)) for n in ("Eta", "U", "V"))
            mc = _interior(cs.get("MASK"))
            cur = ref[start + k + 1]
            wet = ((mask > 0) & (mc > 0)).astype(np.float32)
            xs.append(features(e_in, u_in, v_in, dc, mask))
            tgt = np.stack([cur["Eta"] - ec, cur["U"] - uc, cur["V"] - vc], axis=-1) * OUT_SCALE
            ts.append(np.ascontiguousarray((tgt * wet[..., None]).transpose(1, 0, 2), dtype=np.float32))
            ws.append(np.ascontiguousarray(wet.T))
            e_in, u_in, v_in, mask = ec, uc, vc, mc
    cs.close()
    return np.stack(xs), np.stack(ts), np.stack(ws)


def train(net, x, t, w, iters=400, batch=8, lr=2e-3, seed=0, log=None):
    """Adam on random minibatches of the pairs (all on the GPU).  x, t, w are
    arrays of pairs, or lists of such arrays (one per grid size); a
    minibatch comes from one of them, chosen in proportion to its size."""
    import torch
    dev = torch.device("cuda")
    if not isinstance(x, (list, tuple)):
        x, t, w = [x], [t], [w]
    sets = [(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev), torch.from_numpy(c).to(dev))
            for a, b, c in zip(x, t, w)]
    sizes = np.array([a.shape[0] for a in x], dtype=float)
    rng = np.random.default_rng(seed)
    losses = []
    for it in range(iters):
        X, T, Wm = sets[rng.choice(len(sets), p=sizes / sizes.sum())]
        idx = torch.from_numpy(rng.choice(X.shape[0], size=min(batch, X.shape[0]), replace=False)).to(dev)
        xb, tb, wb = X[idx].contiguous(), T[idx].contiguous(), Wm[idx].contiguous()
        loss = net.loss_grad(xb, tb, wb)
        net.adam(lr * (0.5 ** (it / max(1, iters // 3))))
        losses.append(loss)
        if log and it % 100 == 0:
            log(it, loss)
    return losses


def one_step_error(net, x, t, w):
    """Masked MSE of the targets without and with the network's prediction
    (in OUT_SCALE units), over all pairs."""
    import torch
    dev = torch.device("cuda")
    e0 = e1 = 0.0
    for k in range(x.shape[0]):
        xb = torch.from_numpy(x[k:k + 1]).to(dev).contiguous()
        y = net.forward(xb).cpu().numpy()[0]
        m = w[k][..., None]
        e0 += float(np.sum(m * t[k] ** 2))
        e1 += float(np.sum(m * (t[k] - y) ** 2))
    return e0, e1


def rollout(case, nsteps_c, net=None, precision="MIXED", max_corr=0.2, snaps=()):
    """The coarse twin of case run for nsteps_c steps, with the network's
    correction after every step when net is given; returns (coarse solver
    state dict of interior Eta, U, V, HeightMax, in "snaps" the interior Eta
    and MASK after each step count of snaps and in "rejected" the steps whose
    correction each check rejected; steps corrected)."""
    pf, depth, phases = case
    pc, depth_c = coarse_case(with_defaults(pf), depth)
    pc = with_defaults(pc)
    pc["OUT_Hmax"] = True
    cs = Solver(pc, precision=precision)
    cs.init(depth_c, phases=phases)
    applied = 0
    taken = {}
    # steps whose correction each check rejected (several may reject one)
    rejected = {"size": 0, "drift": 0, "shore": 0, "nonfinite": 0}
    for k in range(nsteps_c):
        cs.step(1)
        if net is not None:
            ok = net.correct(cs, max_corr)
            applied += int(ok)
            if not ok:
                c = net.last_check()
                finite = all(np.isfinite([c["mean_eta"], c["max_abs"]]))
                rejected["nonfinite"] += int(not finite)
                rejected["size"] += int(finite and c["max_abs"] > max_corr)
                rejected["drift"] += int(finite and abs(c["mean_eta"]) > 0.5 * max_corr)
                rejected["shore"] += int(c["dry_m"] > 0.0)
        if k + 1 in snaps:
            taken[k + 1] = (_interior(cs.get("Eta")), _interior(cs.get("MASK")))
    out = {n: _interior(cs.get(n)) for n in ("Eta", "U", "V", "HeightMax", "MASK")}
    out["snaps"] = taken
    out["rejected"] = rejected
    out["TIME"] = cs.scalar("TIME")
    out["depth"] = depth_c
    cs.close()
    return out, applied


def fine_run(case, nsteps_f, precision="MIXED", snaps=()):
    """The fine case run for nsteps_f steps; the state dict as rollout's,
    "snaps" holding the interior Eta and MASK after each step count of
    snaps."""
    pf, depth, phases = case
    pf = with_defaults(pf)
    pf["OUT_Hmax"] = True
    fs = Solver(pf, precision=precision)
    fs.init(depth, phases=phases)
    taken, done = {}, 0
    for k in sorted(set(snaps) | {nsteps_f}):
        if k > nsteps_f:
            break
        fs.step(k - done)
        done = k
        if k in snaps:
            taken[k] = (_interior(fs.get("Eta")), _interior(fs.get("MASK")))
    out = {n: _interior(fs.get(n)) for n in ("Eta", "U", "V", "HeightMax", "MASK")}
    out["snaps"] = taken
    out["TIME"] = fs.scalar("TIME")
    out["depth"] = depth
    fs.close()
    return out
