"""The exchange steps of a run decomposed over ranks (funwave-tvd_gb300/
decomp.py), among gloo ranks on the CPU at 127.0.0.1: the reference's block
ranges, PHI_EXCH's ghost exchange (parallel.F:55-169), the time step's
global minimum (misc.F:277), the pipelined Thomas sweep across ranks
(TRIDx / TRIDy, tridiagnal.F:413-578), which equals the serial sweep
(TRIDx_ser, tridiagnal.F:375-398) bit for bit, and the reduced-system solve
across ranks, which equals it to rounding.  Every rank builds the same
seeded global arrays and checks its own part against them."""
import importlib.util
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "funwave-tvd_gb300")


def _decomp():
    spec = importlib.util.spec_from_file_location("fw_decomp", os.path.join(PKG, "decomp.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _system(L, n, seed):
    """Rows a x(k-1) + x(k) + c x(k+1) = d like the dispersive u/v recovery
    (|a|, |c| <= 0.3), some with a = 0 (dry or masked cells)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(-0.3, 0.3, (L, n))
    c = rng.uniform(-0.3, 0.3, (L, n))
    d = rng.normal(size=(L, n))
    a[rng.random((L, n)) < 0.05] = 0.0
    return a, c, d


def _work(rank, ws, port, q, case):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    D = _decomp()
    g = D.NGHOST
    try:
        dist.init_process_group("gloo")
        M, N, px, py, periodic = case
        t = D.Tile(M, N, px, py, rank, periodic_y=periodic)
        out = {}
        # halo exchange: the ghosts of internal edges come from the global
        # array; ghosts at the grid's edge keep the value they had
        rng = np.random.default_rng(3)
        glob = rng.normal(size=(M + 2 * g, N + 2 * g))
        if periodic:
            # what the ghosts must be: the periodic copy in y
            glob[:, :g] = glob[:, N:N + g]
            glob[:, N + g:] = glob[:, g:2 * g]
        loc = t.local(glob)
        want = loc.copy()
        loc[:g, :] = -7.0 if t.west is not None else loc[:g, :]
        loc[-g:, :] = -7.0 if t.east is not None else loc[-g:, :]
        loc[:, :g] = -7.0 if t.south is not None else loc[:, :g]
        loc[:, -g:] = -7.0 if t.north is not None else loc[:, -g:]
        D.halo_exchange(t, loc)
        out["halo"] = bool(np.array_equal(loc, want))
        # the global minimum of a per-rank value
        out["min"] = D.allreduce_min(10.0 + rank) == 10.0
        # tridiagonal lines across ranks: x lines (one per j) over this
        # rank's row of ranks, y lines over its column
        a, c, d = _system(M, N, 11)
        xs = D.trid_serial(a, c, d)
        i0, i1, j0, j1 = t.i0 - 1, t.i1, t.j0 - 1, t.j1
        xp = D.trid_x_pipelined(t, a[i0:i1, j0:j1], c[i0:i1, j0:j1], d[i0:i1, j0:j1])
        out["trid_x_pipelined"] = bool(np.array_equal(xp, xs[i0:i1, j0:j1]))
        xr = D.trid_x_partitioned(t, a[i0:i1, j0:j1], c[i0:i1, j0:j1], d[i0:i1, j0:j1])
        out["trid_x_partitioned"] = float(np.abs(xr - xs[i0:i1, j0:j1]).max())
        ay, cy, dy = (v.T for v in _system(N, M, 12))  # (M, N): y lines along axis 1
        ys = D.trid_serial(ay.T, cy.T, dy.T).T
        yp = D.trid_y_pipelined(t, ay[i0:i1, j0:j1], cy[i0:i1, j0:j1], dy[i0:i1, j0:j1])
        out["trid_y_pipelined"] = bool(np.array_equal(yp, ys[i0:i1, j0:j1]))
        yr = D.trid_y_partitioned(t, ay[i0:i1, j0:j1], cy[i0:i1, j0:j1], dy[i0:i1, j0:j1])
        out["trid_y_partitioned"] = float(np.abs(yr - ys[i0:i1, j0:j1]).max())
        dist.destroy_process_group()
        q.put((rank, out))
    except Exception as e:  # report to the parent instead of hanging it
        q.put((rank, {"error": repr(e)}))


@pytest.mark.parametrize("case", [(23, 17, 2, 2, False), (30, 13, 3, 1, False), (12, 26, 1, 2, True),
                                  (19, 21, 2, 2, True), (25, 20, 3, 2, True)])
def test_decomposed_exchange_steps(case):
    torch = pytest.importorskip("torch")
    M, N, px, py, _ = case
    ws = px * py
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_work, args=(r, ws, port, q, case)) for r in range(ws)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=180) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    for rank, r in out:
        assert "error" not in r, (rank, r)
        assert r["halo"] and r["min"], (rank, r)
        assert r["trid_x_pipelined"] and r["trid_y_pipelined"], (rank, r)
        assert r["trid_x_partitioned"] <= 1e-13 and r["trid_y_partitioned"] <= 1e-13, (rank, r)


def test_block_ranges_cover_the_grid():
    D = _decomp()
    for n, p in ((2048, 7), (10, 3), (5, 5), (250, 4)):
        ranges = [D.grid_range(1, n, p, r) for r in range(p)]
        assert ranges[0][0] == 1 and ranges[-1][1] == n
        assert all(ranges[k][1] + 1 == ranges[k + 1][0] for k in range(p - 1))
        sizes = [e - s + 1 for s, e in ranges]
        assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
