"""One 1D single-phase domain split into contiguous slabs, one per process (GPU).

The reference advances its domain with a thread pool over the cells
(main.jl:206, 221). Decomposed, rank r owns a contiguous range of the global cells
and holds one ghost cell past each inner end of it (its neighbour's boundary cell).
One step of main.jl:202-241 is then

1. ``local_max``: the max wave speed over the rank's cells;
2. a max-allreduce of those values: the global max, exactly the single-domain one;
3. ``step(global max)``: dt = cfl dx / max (main.jl:212), owned cells updated, ghosts
   held; the global end cells keep the configuration's boundary rule;
4. the halo exchange: each rank sends its first owned cell's record to its left
   neighbour and its last to its right one, which store them as their ghosts.

Every face sees the two cell states it sees in one domain and the max is exact, so
with the global dx the decomposed run is bitwise the single-domain run. The steps
are written against a small stepper interface (``local_max``, ``step``,
``get_cells``, ``set_cells``) and a communicator (``allreduce_max``,
``exchange``), so the same orchestration drives the CUDA slabs (``GpuSlab``) over
torch.distributed (NCCL or gloo) or in one process.
"""
import numpy as np

from . import _lib as L
from .solver import Solver


def owned_range(n_cells, world, rank):
    """Global cells [lo, hi) that rank owns: contiguous, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world or n_cells < 3 * world:
        raise ValueError(f"cannot split {n_cells} cells over {world} ranks")
    base, extra = divmod(n_cells, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def slab_layout(n_cells, world, rank):
    """(first global cell of the slab, slab cells, left ghost, right ghost): the owned
    range widened by one ghost cell at each end that has a neighbour."""
    lo, hi = owned_range(n_cells, world, rank)
    left, right = rank > 0, rank < world - 1
    return lo - int(left), (hi - lo) + int(left) + int(right), left, right


class GpuSlab:
    """A single-phase Solver context as one slab (hyp_set_slab)."""

    def __init__(self, eos, n_global, world, rank, flux="rusanov", bc="frozen", precision="fp64", X=1.0, cfl=0.5):
        self.first, self.n, self.left, self.right = slab_layout(n_global, world, rank)
        self.solver = Solver(eos, self.n, flux=flux, bc=bc, precision=precision, X=X, cfl=cfl)
        h = self.solver._h
        L.check(L.load().hyp_set_slab(h, float(X) / float(n_global), int(self.left), int(self.right)), h, "hyp_set_slab")
        b = L.ctypes.c_int(0)
        L.check(L.load().hyp_cell_record_size(h, L.ctypes.byref(b)), h, "hyp_cell_record_size")
        self.record_dtype = np.float32 if b.value == 128 else np.float64
        self.record_rows = b.value // np.dtype(self.record_dtype).itemsize

    def upload(self, Q_global, t0=0.0):
        """This slab's cells (ghosts included) of a global SoA state."""
        self.solver.upload(np.ascontiguousarray(Q_global[:, self.first:self.first + self.n]), t0)

    def download_owned(self):
        Q = self.solver.download()
        return Q[:, int(self.left):self.n - int(self.right)]

    def local_max(self):
        v = L.ctypes.c_double(0.0)
        h = self.solver._h
        L.check(L.load().hyp_slab_local_max(h, L.ctypes.byref(v)), h, "hyp_slab_local_max")
        return v.value

    def step(self, lam_max):
        t = L.ctypes.c_double(0.0)
        h = self.solver._h
        L.check(L.load().hyp_slab_step(h, float(lam_max), L.ctypes.byref(t)), h, "hyp_slab_step")
        return t.value

    def get_cells(self, first, count=1):
        rec = np.empty((self.record_rows, count), dtype=self.record_dtype)
        h = self.solver._h
        L.check(L.load().hyp_get_cells(h, int(first), int(count), rec.ctypes.data), h, "hyp_get_cells")
        return rec

    def set_cells(self, first, rec):
        rec = np.ascontiguousarray(rec, dtype=self.record_dtype)
        h = self.solver._h
        L.check(L.load().hyp_set_cells(h, int(first), rec.shape[1], rec.ctypes.data), h, "hyp_set_cells")

    def close(self):
        self.solver.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def halo_out(stepper):
    """Records this slab sends: {'left': its first owned cell, 'right': its last}."""
    out = {}
    if stepper.left:
        out["left"] = stepper.get_cells(1)
    if stepper.right:
        out["right"] = stepper.get_cells(stepper.n - 2)
    return out


def halo_in(stepper, from_left, from_right):
    """Store the neighbours' records as this slab's ghosts."""
    if stepper.left:
        stepper.set_cells(0, from_left)
    if stepper.right:
        stepper.set_cells(stepper.n - 1, from_right)


class TorchComm:
    """torch.distributed communicator (gloo: host tensors; NCCL: the records staged on
    the rank's GPU). Ranks are neighbours in rank order."""

    def __init__(self, dist, device=None):
        self.dist, self.device = dist, device
        self.rank, self.world = dist.get_rank(), dist.get_world_size()

    def _t(self, a):
        import torch
        t = torch.from_numpy(np.ascontiguousarray(a))
        return t.to(self.device) if self.device is not None else t

    def allreduce_max(self, x):
        t = self._t(np.array([x], dtype=np.float64))
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.cpu().numpy()[0])

    def exchange(self, out, shape, dtype):
        """Send out['left'] to rank - 1 and out['right'] to rank + 1; return the records
        received from the left and right neighbours (None where there is none)."""
        ops, recv = [], {}
        if self.rank > 0:
            recv["left"] = self._t(np.empty(shape, dtype=dtype))
            ops.append(self.dist.P2POp(self.dist.isend, self._t(out["left"]), self.rank - 1))
            ops.append(self.dist.P2POp(self.dist.irecv, recv["left"], self.rank - 1))
        if self.rank < self.world - 1:
            recv["right"] = self._t(np.empty(shape, dtype=dtype))
            ops.append(self.dist.P2POp(self.dist.isend, self._t(out["right"]), self.rank + 1))
            ops.append(self.dist.P2POp(self.dist.irecv, recv["right"], self.rank + 1))
        if ops:
            for r in self.dist.batch_isend_irecv(ops):
                r.wait()
        return tuple(recv[k].cpu().numpy() if k in recv else None for k in ("left", "right"))


def exchange_halos(stepper, comm):
    out = halo_out(stepper)
    fl, fr = comm.exchange(out, (stepper.record_rows, 1), stepper.record_dtype)
    halo_in(stepper, fl, fr)


def step_decomposed(stepper, comm):
    """One step of the decomposed run on this rank; returns the new time."""
    lam = comm.allreduce_max(stepper.local_max())
    t = stepper.step(lam)
    exchange_halos(stepper, comm)
    return t


def step_all(steppers):
    """One step of every slab of a decomposition held in one process (rank order):
    the same phases as step_decomposed, with the allreduce and the exchange done in place."""
    lam = max(s.local_max() for s in steppers)
    ts = [s.step(lam) for s in steppers]
    outs = [halo_out(s) for s in steppers]
    for r, s in enumerate(steppers):
        halo_in(s, outs[r - 1]["right"] if r > 0 else None, outs[r + 1]["left"] if r + 1 < len(steppers) else None)
    return ts


# ---- a batch's problems over ranks --------------------------------------------------
# The problems of a batch are independent (each its own dx, CFL dt and time:
# main.jl:202-227 per problem), so ranks step disjoint sets of them as separate
# batches with no exchange between steps; only the final states are gathered.

def shard_problems(sizes, world):
    """The problems of a batch (cell counts `sizes`) dealt to `world` ranks so that
    their cell counts balance: largest problem first onto the rank with the fewest cells
    so far (ties to the lower rank, then the lower problem index). Returns one array of
    problem indices per rank, in batch order. No rank's cells exceed the mean by more
    than the largest problem."""
    import heapq
    sizes = np.asarray(sizes, dtype=np.int64)
    if world < 1 or len(sizes) < world or np.any(sizes < 1):
        raise ValueError(f"cannot deal {len(sizes)} problems to {world} ranks")
    order = sorted(range(len(sizes)), key=lambda p: (-int(sizes[p]), p))
    heap = [(0, r) for r in range(world)]
    shards = [[] for _ in range(world)]
    for p in order:
        load, r = heapq.heappop(heap)
        shards[r].append(p)
        heapq.heappush(heap, (load + int(sizes[p]), r))
    return [np.array(sorted(s), dtype=np.int64) for s in shards]


def shard_columns(sizes, problems):
    """Columns of the listed problems in the batch's SoA state (problem p in columns
    offsets[p]:offsets[p + 1]), in the order listed: a shard's own state."""
    offsets = np.concatenate([[0], np.cumsum(np.asarray(sizes, dtype=np.int64))])
    parts = [np.arange(offsets[p], offsets[p + 1]) for p in problems]
    return np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)


def gather_shards(sizes, shards, states):
    """The batch's SoA state from the ranks' shard states (states[r] over the columns
    shard_columns(sizes, shards[r]))."""
    total = int(np.sum(sizes))
    Q = np.empty((states[0].shape[0], total), dtype=states[0].dtype)
    for problems, Qr in zip(shards, states):
        Q[:, shard_columns(sizes, problems)] = Qr
    return Q
