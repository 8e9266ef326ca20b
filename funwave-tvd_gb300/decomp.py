"""Domain decomposition of one run over CPU ranks (torch.distributed, gloo).

The reference runs one domain over MPI ranks: each rank owns a block of the
grid with a ring of Nghost ghost cells (misc.F:100-178, the block ranges of
grid_range_per_procs misc.F:181-204), fills the ghosts of its internal edges
from its neighbours once per stage (PHI_EXCH, parallel.F:55-169), takes the
minimum time step over all ranks (ESTIMATE_DT's MPI_ALLREDUCE, misc.F:277)
and solves the tridiagonal lines that cross rank boundaries by a Thomas
sweep pipelined from rank to rank (TRIDx / TRIDy, tridiagnal.F:413-578).

Every GPU host of this build has one GPU, so a run is never split across
GPUs: this module is the algorithm of those exchange steps, restated on the
host and tested among CPU ranks, as the reference for a decomposed
multi-GPU run.  It holds:
  - Tile: the reference's rank layout, block ranges and neighbours;
  - halo_exchange: PHI_EXCH's east-west then north-south ghost exchange;
  - allreduce_min: the time step's global minimum;
  - trid_x_pipelined / trid_y_pipelined: the reference's pipelined Thomas,
    which performs the serial sweep's operations in the serial order, so
    its result equals trid_serial bit for bit;
  - trid_x_partitioned / trid_y_partitioned: the reduced-system
    (partitioned) solve a GPU decomposition would use instead: each rank reduces its segment of a
    line to two boundary unknowns, the ranks exchange those rows, and each
    rank recovers its segment; equal to the serial solve to rounding.
Arrays are numpy (Mloc, Nloc) with index (i, j), i the x direction, as
the reference's PHI(Mloc, Nloc).
"""
import numpy as np

NGHOST = 3


def grid_range(n1, n2, nprocs, myid):
    """First and last global index of rank myid's block of n1..n2
    (misc.F:181-204): equal blocks, the remainder one each to the first
    ranks."""
    inum1 = (n2 - n1 + 1) // nprocs
    inum2 = (n2 - n1 + 1) % nprocs
    stag = myid * inum1 + n1 + min(myid, inum2)
    endg = stag + inum1 - 1
    if inum2 > myid:
        endg += 1
    return stag, endg


class Tile:
    """Rank `rank`'s block of an Mglob x Nglob grid split PX x PY.  Ranks
    are numbered with the x index outer (ProcessorID(I, J), misc.F:103-114):
    rank = ix * PY + jy.  Neighbours are None at the grid's edge, except in
    y when periodic."""

    def __init__(self, Mglob, Nglob, px, py, rank, periodic_y=False):
        self.Mglob, self.Nglob, self.px, self.py, self.rank = Mglob, Nglob, px, py, rank
        self.ix, self.jy = divmod(rank, py)
        self.i0, self.i1 = grid_range(1, Mglob, px, self.ix)   # 1-based global interior range
        self.j0, self.j1 = grid_range(1, Nglob, py, self.jy)
        self.Mloc = self.i1 - self.i0 + 1 + 2 * NGHOST
        self.Nloc = self.j1 - self.j0 + 1 + 2 * NGHOST

        def at(ix, jy):
            if not 0 <= ix < px:
                return None
            if not 0 <= jy < py:
                # periodic y wraps to the other end; with one rank in y that
                # is this rank, whose ghosts the serial periodic copy fills
                if not periodic_y or py == 1:
                    return None
                jy %= py
            return ix * py + jy

        self.west, self.east = at(self.ix - 1, self.jy), at(self.ix + 1, self.jy)
        self.south, self.north = at(self.ix, self.jy - 1), at(self.ix, self.jy + 1)
        # the neighbours along a line of the tridiagonal solves, which end at
        # the grid's edge in y even when the ghosts wrap
        self.line_south = self.south if self.jy > 0 else None
        self.line_north = self.north if self.jy < py - 1 else None

    def local(self, glob):
        """This rank's (Mloc, Nloc) window of a global array that has the
        global ghost ring: interior and ghosts as the global array holds
        them."""
        g = NGHOST
        return np.array(glob[self.i0 - 1:self.i1 + 2 * g, self.j0 - 1:self.j1 + 2 * g])

    def interior(self, loc):
        g = NGHOST
        return loc[g:-g, g:-g]


def _exchange(dist, send, recv, torch):
    """Post every receive and send (peer, tag, array), wait for all.  The
    send buffers are held until the waits end."""
    reqs, bufs, outs = [], [], []
    for peer, tag, shape in recv:
        b = torch.empty(shape, dtype=torch.float64)
        bufs.append(b)
        reqs.append(dist.irecv(b, src=peer, tag=tag))
    for peer, tag, arr in send:
        t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64))
        outs.append(t)
        reqs.append(dist.isend(t, dst=peer, tag=tag))
    for r in reqs:
        r.wait()
    return [b.numpy() for b in bufs]


def halo_exchange(tile, phi):
    """PHI_EXCH (parallel.F:55-169) in place: the east-west ghost columns of
    every row from the west and east neighbours' first and last Nghost
    interior columns, then the north-south ghost rows of every column,
    corners included, from the south and north neighbours.  Ghosts at the
    grid's edge are left as they are."""
    import torch
    import torch.distributed as dist
    g = NGHOST
    ib, ie = g, phi.shape[0] - g - 1
    jb, je = g, phi.shape[1] - g - 1
    # east-west: tag 0 travels west -> east's west ghosts, tag 1 east -> west
    send, recv = [], []
    if tile.west is not None:
        recv.append((tile.west, 0, (g, phi.shape[1])))
        send.append((tile.west, 1, phi[ib:ib + g, :]))
    if tile.east is not None:
        recv.append((tile.east, 1, (g, phi.shape[1])))
        send.append((tile.east, 0, phi[ie - g + 1:ie + 1, :]))
    got = _exchange(dist, send, recv, torch)
    k = 0
    if tile.west is not None:
        phi[ib - g:ib, :] = got[k]
        k += 1
    if tile.east is not None:
        phi[ie + 1:ie + 1 + g, :] = got[k]
    # north-south over every column, the x ghosts just filled included
    send, recv = [], []
    if tile.south is not None:
        recv.append((tile.south, 2, (phi.shape[0], g)))
        send.append((tile.south, 3, phi[:, jb:jb + g]))
    if tile.north is not None:
        recv.append((tile.north, 3, (phi.shape[0], g)))
        send.append((tile.north, 2, phi[:, je - g + 1:je + 1]))
    got = _exchange(dist, send, recv, torch)
    k = 0
    if tile.south is not None:
        phi[:, jb - g:jb] = got[k]
        k += 1
    if tile.north is not None:
        phi[:, je + 1:je + 1 + g] = got[k]
    return phi


def allreduce_min(x):
    """The global minimum of a per-rank value (ESTIMATE_DT, misc.F:277)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MIN)
    return float(t.item())


def trid_serial(a, c, d):
    """TRIDx_ser (tridiagnal.F:375-398) along axis 0 of (L, nlines) arrays:
    rows a_k x_(k-1) + x_k + c_k x_(k+1) = d_k, the elimination skipped
    where a_k = 0.  Returns x; a, c, d are not modified."""
    c, d = np.array(c, dtype=np.float64), np.array(d, dtype=np.float64)
    L = c.shape[0]
    for k in range(1, L):
        nz = a[k] != 0.0
        den = 1.0 / a[k, nz] - c[k - 1, nz]
        c[k, nz] = c[k, nz] / a[k, nz] / den
        d[k, nz] = (d[k, nz] / a[k, nz] - d[k - 1, nz]) / den
    x = np.empty_like(d)
    x[L - 1] = d[L - 1]
    for k in range(L - 2, -1, -1):
        x[k] = d[k] - c[k] * x[k + 1]
    return x


def _trid_pipelined(a, c, d, prev, nxt, tag):
    """TRIDx (tridiagnal.F:413-488) on this rank's segment of every line
    (axis 0 the line, interior rows only): the previous rank's last (d, c)
    enters the first row, the sweep runs, the last (d, c) goes on; back
    substitution receives the next rank's first x and sends its own back."""
    import torch
    import torch.distributed as dist
    c, d = np.array(c, dtype=np.float64), np.array(d, dtype=np.float64)
    L, n = c.shape
    if prev is not None:
        dc = _exchange(dist, [], [(prev, tag, (2, n))], torch)[0]
        nz = a[0] != 0.0
        den = 1.0 / a[0, nz] - dc[1, nz]
        c[0, nz] = c[0, nz] / a[0, nz] / den
        d[0, nz] = (d[0, nz] / a[0, nz] - dc[0, nz]) / den
    for k in range(1, L):
        nz = a[k] != 0.0
        den = 1.0 / a[k, nz] - c[k - 1, nz]
        c[k, nz] = c[k, nz] / a[k, nz] / den
        d[k, nz] = (d[k, nz] / a[k, nz] - d[k - 1, nz]) / den
    if nxt is not None:
        _exchange(dist, [(nxt, tag, np.stack([d[L - 1], c[L - 1]]))], [], torch)
    x = np.empty_like(d)
    if nxt is not None:
        xn = _exchange(dist, [], [(nxt, tag + 1, (1, n))], torch)[0][0]
        x[L - 1] = d[L - 1] - c[L - 1] * xn
    else:
        x[L - 1] = d[L - 1]
    for k in range(L - 2, -1, -1):
        x[k] = d[k] - c[k] * x[k + 1]
    if prev is not None:
        _exchange(dist, [(prev, tag + 1, x[0:1])], [], torch)
    return x


def trid_x_pipelined(tile, a, c, d):
    """The x lines of the interior (local interior arrays (Mint, Nint)) solved
    across the ranks of this tile's row of ranks, west to east."""
    return _trid_pipelined(a, c, d, tile.west, tile.east, 10)


def trid_y_pipelined(tile, a, c, d):
    """The y lines (TRIDy, tridiagnal.F:502-578), south to north."""
    return _trid_pipelined(a.T, c.T, d.T, tile.line_south, tile.line_north, 20).T


def _segment_parts(a, c, d):
    """One rank's segment of each line (axis 0), the couplings to the
    unknowns outside it kept apart: x_k = y_k - v_k x_left - w_k x_right, with
    T y = d, T v = a_0 e_0, T w = c_last e_last, T the segment's own rows
    (the first row's a and the last row's c taken out)."""
    L = a.shape[0]
    e0 = np.zeros_like(d)
    e0[0] = a[0]
    eL = np.zeros_like(d)
    eL[L - 1] = c[L - 1]
    aa, cc = np.array(a, dtype=np.float64), np.array(c, dtype=np.float64)
    aa[0] = 0.0
    cc[L - 1] = 0.0
    # one elimination for the three right-hand sides
    rhs = np.stack([d, e0, eL])           # (3, L, n)
    cp = np.empty_like(cc)
    cp[0] = cc[0]
    r = np.array(rhs)
    for k in range(1, L):
        den = 1.0 - aa[k] * cp[k - 1]
        cp[k] = cc[k] / den
        r[:, k] = (rhs[:, k] - aa[k] * r[:, k - 1]) / den
    x = np.empty_like(r)
    x[:, L - 1] = r[:, L - 1]
    for k in range(L - 2, -1, -1):
        x[:, k] = r[:, k] - cp[k] * x[:, k + 1]
    return x[0], x[1], x[2]


def trid_x_partitioned(tile, a, c, d):
    """The x lines solved by the reduced system: each rank reduces its
    segment to the rows of its first and last unknowns, all ranks of the
    row gather those rows, solve the reduced system of 2 P unknowns per
    line, and recover their segments."""
    row = [ix * tile.py + tile.jy for ix in range(tile.px)]  # the ranks sharing these lines, west to east
    return _partitioned(tile, a, c, d, row, 30)


def trid_y_partitioned(tile, a, c, d):
    """The y lines (non-periodic) by the reduced system over this tile's
    column of ranks, south to north."""
    col = [tile.ix * tile.py + jy for jy in range(tile.py)]
    return _partitioned(tile, a.T, c.T, d.T, col, 40).T


def _partitioned(tile, a, c, d, row, tag0):
    """The reduced-system solve of the lines along axis 0 of this rank's
    segments, over the ranks of row (in line order)."""
    import torch
    import torch.distributed as dist
    y, v, w = _segment_parts(a, c, d)
    L, n = y.shape
    mine = np.stack([y[0], v[0], w[0], y[L - 1], v[L - 1], w[L - 1]])  # (6, n)
    parts = []
    for r in row:
        if r == tile.rank:
            parts.append(mine)
        else:
            parts.append(None)
    # every rank of the row sends its rows to every other one
    send = [(r, tag0 + tile.rank, mine) for r in row if r != tile.rank]
    recv = [(r, tag0 + r, (6, n)) for r in row if r != tile.rank]
    got = _exchange(dist, send, recv, torch)
    k = 0
    for i, r in enumerate(row):
        if r != tile.rank:
            parts[i] = got[k]
            k += 1
    P = len(row)
    # unknowns s_0, e_0, s_1, e_1, ...: s_p = y - v e_(p-1) - w s_(p+1),
    # e_p = y' - v' e_(p-1) - w' s_(p+1)
    xs = np.empty((2 * P, n))
    for line in range(n):
        M = np.eye(2 * P)
        rhs = np.empty(2 * P)
        for p in range(P):
            ys, vs, ws, ye, ve, we = parts[p][:, line]
            for off, (yy, vv, ww) in enumerate(((ys, vs, ws), (ye, ve, we))):
                q = 2 * p + off
                rhs[q] = yy
                if p > 0:
                    M[q, 2 * p - 1] += vv
                if p < P - 1:
                    M[q, 2 * p + 2] += ww
        xs[:, line] = np.linalg.solve(M, rhs)
    p = row.index(tile.rank)
    left = xs[2 * p - 1] if p > 0 else np.zeros(n)
    right = xs[2 * p + 2] if p < P - 1 else np.zeros(n)
    return y - v * left - w * right
