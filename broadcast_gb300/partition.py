"""Domain decomposition of one grid over several ranks (one GPU each).

The grid is cut into slabs of whole columns i (i is the fastest axis of the
reference's Fortran layout).  Each rank holds its slab with gh = 3 halo
columns on both sides and the full j extent (ghost rows included), in the
same padded Fortran layout as a whole grid, so the unmodified residual, tangent
and boundary kernels run on it: the DNC5 residual has no special i rows (its
near-boundary rows are in j), and every boundary fill acts on one column or
row at a time.

  ColumnSlabs   : column ranges per rank, extraction of a slab from global
                  arrays and insertion of its owned columns back;
  HaloExchange  : before each residual / tangent evaluation, the gh + 1
                  edge columns go to the neighbouring ranks (and, for the
                  periodic O-mesh, between the first and last rank, replacing
                  jn_match_2d); every wait is bounded by `timeout` seconds and a
                  missing neighbour raises HaloTimeout instead of hanging;
  global_norml2 : the L2 residual norm (srcfv/norm.F90:2) as a sum-allreduce
                  of the per-slab sums of squares.

Ranks exchange through torch.distributed point-to-point calls (NCCL between
GPUs, gloo between CPU processes).  No collective runs on the data path other
than the halo exchange and the norm reduction.
"""
import datetime

import numpy as np

GH = 3


class HaloTimeout(RuntimeError):
    """A neighbouring rank did not deliver its halo within the time limit."""


class ColumnSlabs:
    """Partition of the interior columns 1..im into `nranks` contiguous slabs.

    A slab's local grid is its owned columns plus `overlap` columns on every
    side that has a neighbour (computed again, results discarded), plus gh
    halo columns.  The overlap is needed because the residual extrapolates
    the velocity gradients of the Ducros sensor into ghost columns
    (rhs/gradveloingh.F) instead of computing them: with one overlap column
    the faces of the owned columns see computed gradients only.  Halo
    exchanges therefore move gh + overlap columns.  `periodic` joins column
    im to column 1 (the O-mesh), so every slab has two neighbours."""

    def __init__(self, im, jm, nranks, gh=GH, periodic=False, overlap=1):
        if nranks < 1:
            raise ValueError("nranks must be >= 1")
        if im < nranks * (gh + overlap + 1):
            raise ValueError("each slab needs at least gh + overlap + 1 = %d columns" % (gh + overlap + 1))
        self.im, self.jm, self.nranks, self.gh = im, jm, nranks, gh
        self.periodic, self.overlap = periodic, overlap
        base, extra = divmod(im, nranks)
        self.ranges = []
        i0 = 1
        for r in range(nranks):
            n = base + (1 if r < extra else 0)
            self.ranges.append((i0, i0 + n - 1))
            i0 += n

    def owned(self, rank):
        """(first, last) global interior column of `rank`, 1-based inclusive."""
        return self.ranges[rank]

    def has_left(self, rank):
        return self.nranks > 1 and (rank > 0 or self.periodic)

    def has_right(self, rank):
        return self.nranks > 1 and (rank < self.nranks - 1 or self.periodic)

    def overlaps(self, rank):
        return (self.overlap if self.has_left(rank) else 0, self.overlap if self.has_right(rank) else 0)

    def local_im(self, rank):
        a, b = self.ranges[rank]
        ol, orr = self.overlaps(rank)
        return b - a + 1 + ol + orr

    def _columns(self, rank, extra):
        """Global padded-array positions (0-based) of the slab's local columns
        (+ `extra` for node arrays).  Columns beyond 1..im wrap when periodic."""
        a, b = self.ranges[rank]
        ol, orr = self.overlaps(rank)
        g = self.gh
        cols = np.arange(a - ol - g, b + orr + g + 1 + extra)  # global 1-based column indices
        if self.periodic and self.nranks > 1:
            inner = (cols >= 1) & (cols <= self.im + extra)
            cols = np.where(inner, cols, (cols - 1) % self.im + 1)
        return cols - 1 + g

    def extract_cells(self, a, rank):
        """Slab of a padded cell array (im+2gh, jm+2gh[, ...]) -> (im_loc+2gh, jm+2gh[, ...])."""
        return np.asfortranarray(np.take(a, self._columns(rank, 0), axis=0))

    def extract_nodes(self, a, rank):
        """Slab of a padded node array (im+2gh+1, jm+2gh+1[, ...])."""
        return np.asfortranarray(np.take(a, self._columns(rank, 1), axis=0))

    def extract_grid(self, grid, rank):
        """Metrics of the slab, as a grid dictionary for the operator API."""
        out = {k: self.extract_cells(grid[k], rank) for k in ("xc", "yc", "vol", "volf")}
        out.update({k: self.extract_nodes(grid[k], rank) for k in ("x0", "y0", "nx", "ny")})
        out.update(im=self.local_im(rank), jm=self.jm, gh=self.gh)
        return out

    def owned_slice(self, rank):
        """Local column positions (0-based, padded array) of the owned columns."""
        a, b = self.ranges[rank]
        ol, _ = self.overlaps(rank)
        return slice(self.gh + ol, self.gh + ol + b - a + 1)

    def insert_owned(self, local, global_, rank):
        """Write the owned columns (all j, ghost rows included) of a slab back."""
        a, b = self.ranges[rank]
        global_[a - 1 + self.gh:b + self.gh] = local[self.owned_slice(rank)]


class HaloExchange:
    """Halo columns of one rank's slab.

    Works on numpy arrays in Fortran layout (ni_loc, nj, nv) or on torch
    tensors in the operator layout (nv, nj, ni_loc).  `periodic` joins the
    first and last slab (the O-mesh's i direction)."""

    def __init__(self, slabs, rank, timeout=10.0, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.slabs, self.rank = slabs, rank
        self.timeout = float(timeout)
        self.group = group
        n = slabs.nranks
        self.left = (rank - 1) % n if slabs.has_left(rank) else None
        self.right = (rank + 1) % n if slabs.has_right(rank) else None
        self.width = slabs.gh + slabs.overlap  # columns moved per side

    def _cols(self, a, lo, hi):
        import torch
        if isinstance(a, torch.Tensor):
            return a[..., lo:hi]
        return a[lo:hi]

    def exchange(self, a):
        """Fill the halo and overlap columns on both sides from the neighbours
        (in place): the first / last gh + overlap owned columns of the
        neighbour land in this slab's leading / trailing gh + overlap columns."""
        import torch
        wdt = self.width
        ni = (a.shape[-1] if isinstance(a, torch.Tensor) else a.shape[0])
        own = self.slabs.owned_slice(self.rank)
        is_t = isinstance(a, torch.Tensor)
        to_t = (lambda x: x.contiguous().clone()) if is_t else (lambda x: torch.from_numpy(np.ascontiguousarray(x)))
        send_l = to_t(self._cols(a, own.start, own.start + wdt)) if self.left is not None else None
        send_r = to_t(self._cols(a, own.stop - wdt, own.stop)) if self.right is not None else None
        recv_l = torch.empty_like(send_l) if send_l is not None else None
        recv_r = torch.empty_like(send_r) if send_r is not None else None
        # Columns moving right carry tag 1, columns moving left tag 2, and every
        # rank posts in the order (send right, receive from left, send left,
        # receive from right), so that messages pair correctly also when the
        # left and right neighbour are the same rank (two periodic slabs) and
        # on backends that pair by order rather than by tag.
        ops = []
        P2P, d = self.dist.P2POp, self.dist
        if self.right is not None:
            ops.append(P2P(d.isend, send_r, self.right, self.group, 1))
        if self.left is not None:
            ops.append(P2P(d.irecv, recv_l, self.left, self.group, 1))
            ops.append(P2P(d.isend, send_l, self.left, self.group, 2))
        if self.right is not None:
            ops.append(P2P(d.irecv, recv_r, self.right, self.group, 2))
        if not ops:
            return a
        try:
            reqs = self.dist.batch_isend_irecv(ops)
            for r in reqs:
                try:
                    ok = r.wait(datetime.timedelta(seconds=self.timeout))
                except TypeError:  # a backend whose wait takes no time limit: the group's timeout applies
                    ok = r.wait()
                if ok is False:
                    raise HaloTimeout("rank %d: halo not received within %.1f s" % (self.rank, self.timeout))
        except HaloTimeout:
            raise
        except Exception as e:  # the peer closed its connection or the wait timed out
            raise HaloTimeout("rank %d: halo exchange failed (%s)" % (self.rank, e)) from e
        if self.left is not None:
            self._put(a, 0, wdt, recv_l)
        if self.right is not None:
            self._put(a, ni - wdt, ni, recv_r)
        return a

    def _put(self, a, lo, hi, buf):
        import torch
        if isinstance(a, torch.Tensor):
            a[..., lo:hi] = buf.to(a.device)
        else:
            a[lo:hi] = buf.numpy()


def global_norml2(local_sumsq, group=None):
    """sqrt of the sum over ranks of the per-slab sums of squares (5-vector)."""
    import torch
    import torch.distributed as dist
    t = torch.as_tensor(np.asarray(local_sumsq, dtype=np.float64)).clone()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return np.sqrt(t.numpy())
