"""One evolution split over several ranks (GPUs): slab decomposition along i2.

The reference runs one grid in one process (its drivers have no domain
decomposition); this module spreads one method-of-lines evolution of
MoL_step_forward_in_time (MoLtimestepping/C_Code_Generation.py:141-168 and
:266-329: per RK4 substep the RHS and update at interior points, then
apply_bcs_curvilinear, then the BSSN det(gammabar) rescale) over `world`
ranks without changing its arithmetic.

Partition.  The Nxx2 interior planes of i2 (the outermost, contiguous index
of the IDX4S layout) are split into `world` consecutive slabs of at least
max(NGHOSTS, 3) planes; rank r owns interior planes [z0_r, z1_r), the first
rank also the NGHOSTS low ghost planes and the last rank the high ones.
Each rank holds its planes plus NGHOSTS halo planes on each side (the
window [z0_r - NGHOSTS, z1_r + NGHOSTS)) as a grid of its own
(Grid.slab), so the library's interior kernels run unchanged on it.

One substep on every rank:
1. the RHS and RK update at the slab's interior points (MoL_substep_rhs);
2. the boundary conditions at the ghost points the rank owns, ghost layer
   by ghost layer as apply_bcs_curvilinear orders them: the outer rule
   (quadratic extrapolation, whose sources lie in the rank's own planes),
   then the inner parity copies, whose sources can lie on any rank (the phi
   wrap and the theta/r reflections of curvilinear grids map a ghost point
   to a plane far away in i2): each rank gathers the source values others
   request from it, the buffers travel rank to rank, and each rank writes
   its ghost points from what it received;
3. the BSSN rescale at every point of the slab;
4. the halo exchange: each rank sends its NGHOSTS first and last owned
   planes (all gridfunctions, ghost columns included) to its neighbours.
Every point is written by exactly one rank from the same values as in the
one-grid step, so the result is the one-grid result.  Norms over the grid
are the all-reduced sums of squares over each rank's interior points.

The exchange goes through a communicator: `DistComm` (torch.distributed:
NCCL point-to-point between GPUs, or gloo on CPU) with one rank per
process, or `LocalComm`, which drives several ranks in this process (one
GPU; the buffers are handed over, nothing waits on another rank's kernel).
The per-rank operations are those of `LibSlabOps` (libnrgpu kernels, FP64);
the index plan (`SlabPlan`) is plain numpy.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .grid import SYSTEM_GFS, Grid


# ------------------------------------------------------------------ plan
def slab_ranges(Nxx2, NGHOSTS, world):
    """[(z0, z1)] per rank: the interior planes of i2 (NGHOSTS .. NGHOSTS +
    Nxx2 - 1) in consecutive slabs whose sizes differ by at most one."""
    world = int(world)
    if world < 1:
        raise ValueError("world must be >= 1")
    need = max(NGHOSTS, 3)
    if Nxx2 < need * world:
        raise ValueError("Nxx2 = %d planes cannot give %d ranks %d planes each" % (Nxx2, world, need))
    base, rem = divmod(Nxx2, world)
    out, z = [], NGHOSTS
    for r in range(world):
        n = base + (1 if r < rem else 0)
        out.append((z, z + n))
        z += n
    return out


def bcmap_layers(bcmap):
    """Per ghost layer: ([(dest, step) for face directions i0, i1, i2],
    (inner dest, inner src, inner parity bits)) from a boundary map in the
    form of Evolution.bc_map() (global idx3)."""
    layers = []
    for g in range(len(bcmap["num_ob"])):
        ds = bcmap["ob_dir_start"][g]
        outer = [(np.asarray(bcmap["outer_dest"][ds[d]:ds[d + 1]], dtype=np.int64),
                  np.asarray(bcmap["outer_step"][ds[d]:ds[d + 1]], dtype=np.int64)) for d in range(3)]
        a, n = bcmap["ib_start"][g], bcmap["num_ib"][g]
        inner = tuple(np.asarray(bcmap[k][a:a + n], dtype=np.int64) for k in ("inner_dest", "inner_src",
                                                                             "inner_parity"))
        layers.append((outer, inner))
    return layers


class SlabPlan:
    """Rank `rank`'s share of a grid of (n0, n1, n2) points (ghosts
    included) split over `world` ranks, and its exchanges.

    outer[k][d] = (dest, step): the outer points of ghost layer k, face
        direction d, that this rank owns, in slab idx3 (int32);
    inner_dest[k], inner_parity[k]: this rank's inner points of layer k,
        grouped by the rank that owns their source (rank order);
    inner_counts[k][q]: how many of them rank q supplies;
    inner_send[k][q]: slab idx3 of the sources rank q requests from this
        rank, in q's order (q == rank included: the local copies);
    halo_send / halo_recv: {peer: (first plane, end plane)} of the slab.
    """

    def __init__(self, n, NGHOSTS, bcmap, rank, world):
        n0, n1, n2 = (int(v) for v in n)
        ng = int(NGHOSTS)
        self.n, self.ng, self.rank, self.world = (n0, n1, n2), ng, int(rank), int(world)
        ranges = slab_ranges(n2 - 2 * ng, ng, world)
        self.ranges = ranges
        self.z0, self.z1 = ranges[rank]
        self.w0, self.w1 = self.z0 - ng, self.z1 + ng
        self.n2l = self.w1 - self.w0
        plane = n0 * n1
        owner = np.empty(n2, dtype=np.int64)
        for r, (a, b) in enumerate(ranges):
            owner[a:b] = r
        owner[:ng] = 0
        owner[n2 - ng:] = world - 1
        self.owner_of_plane = owner
        w0s = np.array([a - ng for a, _ in ranges], dtype=np.int64)

        def local(idx, r):
            return (idx - w0s[r] * plane).astype(np.int32)

        self.outer, self.inner_dest, self.inner_parity, self.inner_counts, self.inner_send = [], [], [], [], []
        for k, (outer, (idst, isrc, ipar)) in enumerate(bcmap_layers(bcmap)):
            mine = []
            for dest, step in outer:
                own = owner[dest // plane] == rank
                d, s = dest[own], step[own]
                for m in (1, 2, 3):
                    if np.any(owner[(d + m * s) // plane] != rank):
                        raise ValueError("ghost layer %d: an outer point of rank %d extrapolates from another "
                                         "rank's planes (slabs too thin)" % (k, rank))
                mine.append((local(d, rank), s.astype(np.int32)))
            self.outer.append(mine)
            dst_owner = owner[idst // plane]
            src_owner = owner[isrc // plane]
            sel = np.nonzero(dst_owner == rank)[0]
            order = sel[np.argsort(src_owner[sel], kind="stable")]
            self.inner_dest.append(local(idst[order], rank))
            self.inner_parity.append(ipar[order].astype(np.int32))
            self.inner_counts.append([int(np.count_nonzero(src_owner[sel] == q)) for q in range(world)])
            send = {}
            for q in range(world):
                selq = np.nonzero((dst_owner == q) & (src_owner == rank))[0]
                if len(selq) == 0:
                    continue
                # q's order: its inner points grouped by source rank, stable
                send[q] = local(isrc[selq], rank)
            self.inner_send.append(send)
        self.halo_send, self.halo_recv = {}, {}
        if rank > 0:
            self.halo_send[rank - 1] = (ng, 2 * ng)
            self.halo_recv[rank - 1] = (0, ng)
        if rank < world - 1:
            self.halo_send[rank + 1] = (self.n2l - 2 * ng, self.n2l - ng)
            self.halo_recv[rank + 1] = (self.n2l - ng, self.n2l)

    @property
    def owned_planes(self):
        """(first, end) of the planes this rank owns, in slab plane index."""
        a = 0 if self.rank == 0 else self.ng
        b = self.n2l if self.rank == self.world - 1 else self.n2l - self.ng
        return a, b

    @property
    def owned_global(self):
        a, b = self.owned_planes
        return self.w0 + a, self.w0 + b


# ------------------------------------------------------------ communicators
class LocalComm:
    """Every rank in this process: an exchange hands each buffer over."""

    def __init__(self, world):
        self.world = int(world)
        self.ranks = list(range(self.world))

    def exchange(self, sends, recv_specs):
        """sends[p][q]: tensor from rank p to rank q; returns recvs[q][p]."""
        out = {q: {} for q in self.ranks}
        for p, d in sends.items():
            for q, t in d.items():
                out[q][p] = t
        return out

    def allreduce_sum(self, vals):
        tot = None
        for r in self.ranks:
            tot = vals[r].clone() if tot is None else tot + vals[r]
        return {r: tot for r in self.ranks}


class DistComm:
    """One rank per process over torch.distributed (NCCL between GPUs, gloo
    on CPU): point-to-point sends and receives of the sizes the plan gives."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.ranks = [self.rank]

    def exchange(self, sends, recv_specs):
        dist = self.dist
        me = self.rank
        out = {me: {}}
        reqs = []
        nccl = dist.get_backend(self.group) == "nccl"
        ops = []
        for q, t in sends.get(me, {}).items():
            if q == me:
                out[me][me] = t
            elif nccl:
                ops.append(dist.P2POp(dist.isend, t.contiguous(), q, self.group))
            else:
                reqs.append(dist.isend(t.contiguous(), q, self.group))
        for p, (numel, dtype, device) in recv_specs.get(me, {}).items():
            if p == me:
                continue
            buf = torch.empty(numel, dtype=dtype, device=device)
            out[me][p] = buf
            if nccl:
                ops.append(dist.P2POp(dist.irecv, buf, p, self.group))
            else:
                reqs.append(dist.irecv(buf, p, self.group))
        if ops:
            reqs.extend(dist.batch_isend_irecv(ops))
        for r in reqs:
            r.wait()
        return out

    def allreduce_sum(self, vals):
        t = vals[self.rank].clone()
        self.dist.all_reduce(t, group=self.group)
        return {self.rank: t}


# ------------------------------------------------------------- the stepper
class SlabStepper:
    """The RK4 step of a slab-decomposed evolution over the ranks `comm`
    drives, with the per-rank operations of `ops` (see LibSlabOps)."""

    def __init__(self, plans, comm, ops):
        self.plans = plans  # {rank: SlabPlan}
        self.comm = comm
        self.ops = ops
        self._bufs = {}  # exchange buffers, allocated once per (rank, layer, peer)

    def _buffer(self, key, r, n):
        b = self._bufs.get(key)
        if b is None or b.numel() != n:
            b = self.ops.new_buffer(r, n)
            self._bufs[key] = b
        return b

    def step(self, dt):
        for s in range(4):
            for r in self.comm.ranks:
                self.ops.substep(r, s, dt)
            self.apply_bcs(s)
            for r in self.comm.ranks:
                self.ops.post(r, s)
            self.halo(s)

    def apply_bcs(self, s):
        ops, comm = self.ops, self.comm
        ngf = ops.ngf
        any_plan = self.plans[comm.ranks[0]]
        for k in range(len(any_plan.outer)):
            for r in comm.ranks:
                ops.outer(r, s, k)
            sends, specs, recv = {}, {}, {}
            for r in comm.ranks:
                pl = self.plans[r]
                counts = pl.inner_counts[k]
                recv[r] = self._buffer(("recv", r, k), r, sum(counts) * ngf)
                offs = np.concatenate([[0], np.cumsum(counts)]) * ngf
                sends[r] = {}
                for q, idx in pl.inner_send[k].items():
                    if q == r:  # local sources straight into this rank's receive buffer
                        ops.gather(r, s, k, q, recv[r][offs[r]:offs[r + 1]])
                    else:
                        buf = self._buffer(("send", r, k, q), r, len(idx) * ngf)
                        ops.gather(r, s, k, q, buf)
                        sends[r][q] = buf
                specs[r] = {q: (counts[q] * ngf, recv[r].dtype, recv[r].device) for q in range(comm.world)
                            if counts[q] and q != r}
            got = comm.exchange(sends, specs)
            for r in comm.ranks:
                pl = self.plans[r]
                offs = np.concatenate([[0], np.cumsum(pl.inner_counts[k])]) * ngf
                for q, t in got[r].items():
                    if q != r:
                        recv[r][offs[q]:offs[q + 1]].copy_(t.reshape(-1))
                ops.scatter(r, s, k, recv[r])

    def halo(self, s):
        ops, comm = self.ops, self.comm
        sends, specs = {}, {}
        for r in comm.ranks:
            pl = self.plans[r]
            sends[r] = {q: ops.planes(r, s, a, b).contiguous() for q, (a, b) in pl.halo_send.items()}
            t = ops.stage_buffer(r, s)
            specs[r] = {q: (ops.ngf * (b - a) * ops.plane_points, t.dtype, t.device)
                        for q, (a, b) in pl.halo_recv.items()}
        got = comm.exchange(sends, specs)
        for r in comm.ranks:
            pl = self.plans[r]
            for q, (a, b) in pl.halo_recv.items():
                ops.planes(r, s, a, b).copy_(got[r][q].reshape(ops.planes(r, s, a, b).shape))


# ------------------------------------------------------- library operations
class LibSlabOps:
    """Per-rank operations on the GPU: each rank's slab is an Evolution
    (boundary="none") of Grid.slab; every arithmetic operation is a
    libnrgpu kernel (MoL_substep_rhs, nrgpu_bc_outer_points,
    nrgpu_bc_gather_points, nrgpu_bc_scatter_parity,
    BSSN_enforce_detgammabar_constraint); the buffers and the plane copies of
    the halo exchange are torch plumbing."""

    def __init__(self, system, grid, plans, device):
        from .mol import Evolution
        self.lib = _lib.load()
        self.system = system
        self.ngf = len(SYSTEM_GFS[system][0])
        self.plans = plans
        self.device = torch.device(device)
        n0, n1, _ = plans[next(iter(plans))].n
        self.plane_points = n0 * n1
        self.ev, self.dev_plan = {}, {}
        for r, pl in plans.items():
            self.ev[r] = Evolution(system, grid.slab(pl.w0, pl.w1), precision="fp64", device=device,
                                   boundary="none")
            dv = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.int32, device=self.device)
            self.dev_plan[r] = dict(
                outer=[[(dv(d), dv(st), len(d)) for d, st in layer] for layer in pl.outer],
                inner_dest=[dv(a) for a in pl.inner_dest], inner_parity=[dv(a) for a in pl.inner_parity],
                inner_send=[{q: (dv(a), len(a)) for q, a in sendk.items()} for sendk in pl.inner_send])

    def stage_buffer(self, r, s):
        ev = self.ev[r]
        return ev.y_n if s == 3 else (ev.k_odd if s % 2 == 0 else ev.k_even)

    def planes(self, r, s, a, b):
        return self.stage_buffer(r, s)[:, a:b]

    def new_buffer(self, r, n):
        return torch.empty(int(n), dtype=torch.float64, device=self.device)

    def _p(self, r):
        return C.byref(self.ev[r].grid.params)

    def substep(self, r, s, dt):
        ev = self.ev[r]
        ev._sync_stream()
        _lib.check(self.lib.MoL_substep_rhs(ev.sys_id, ev._rfm(), self._p(r), C.byref(ev.gfs), s, float(dt), 0),
                   "MoL_substep_rhs")

    def outer(self, r, s, k):
        buf = self.stage_buffer(r, s)
        for d, st, n in self.dev_plan[r]["outer"][k]:
            if n:
                _lib.check(self.lib.nrgpu_bc_outer_points(self._p(r), self.ngf, _lib.ptr(d), _lib.ptr(st), n,
                                                          _lib.ptr(buf)), "nrgpu_bc_outer_points")

    def gather(self, r, s, k, q, out):
        idx, n = self.dev_plan[r]["inner_send"][k][q]
        _lib.check(self.lib.nrgpu_bc_gather_points(self._p(r), self.ngf, _lib.ptr(idx), n,
                                                   _lib.ptr(self.stage_buffer(r, s)), _lib.ptr(out)),
                   "nrgpu_bc_gather_points")

    def scatter(self, r, s, k, recv):
        dest, par = self.dev_plan[r]["inner_dest"][k], self.dev_plan[r]["inner_parity"][k]
        n = dest.numel()
        if n:
            ev = self.ev[r]
            _lib.check(self.lib.nrgpu_bc_scatter_parity(self._p(r), self.ngf,
                                                        C.cast(ev.parity, C.POINTER(C.c_int8)), _lib.ptr(dest),
                                                        _lib.ptr(par), n, _lib.ptr(recv),
                                                        _lib.ptr(self.stage_buffer(r, s))),
                       "nrgpu_bc_scatter_parity")

    def post(self, r, s):
        if self.system == "BSSN":
            self.ev[r].enforce_detgammabar(self.stage_buffer(r, s))


def download_bcmap(grid: Grid):
    """The boundary map of the whole grid (Evolution.bc_map() form), built on
    the device by driver_bcstruct and copied to the host; no state arrays."""
    lib = _lib.load()
    bc = _lib.bc_struct()
    _lib.check(lib.driver_bcstruct(C.byref(grid.params), C.byref(bc)), "driver_bcstruct")
    try:
        arrs = [np.zeros(max(bc.total_outer, 1), dtype=np.int32) for _ in range(2)] + \
               [np.zeros(max(bc.total_inner, 1), dtype=np.int32) for _ in range(3)]
        _lib.check(lib.bcstruct_download(C.byref(bc), *[a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs]),
                   "bcstruct_download")
        return dict(outer_dest=arrs[0][:bc.total_outer], outer_step=arrs[1][:bc.total_outer],
                    inner_dest=arrs[2][:bc.total_inner], inner_src=arrs[3][:bc.total_inner],
                    inner_parity=arrs[4][:bc.total_inner],
                    num_ob=list(bc.num_ob_gz_pts)[:bc.NGHOSTS], num_ib=list(bc.num_ib_gz_pts)[:bc.NGHOSTS],
                    ob_dir_start=[list(bc.ob_dir_start[g]) for g in range(bc.NGHOSTS)],
                    ib_start=list(bc.ib_start)[:bc.NGHOSTS])
    finally:
        lib.bcstruct_freemem(C.byref(bc))


class SlabEvolution:
    """One FP64 evolution of `system` on `grid`, split along i2 over the ranks
    of `comm` (DistComm: this process's rank; LocalComm: all of them here)."""

    def __init__(self, system, grid: Grid, comm, device="cuda"):
        if system not in SYSTEM_GFS:
            raise ValueError("unknown system %r" % system)
        if system == "BSSN" and grid.params.enable_stress_energy_source_terms:
            raise ValueError("stress-energy source terms are not distributed")
        self.system, self.grid, self.comm = system, grid, comm
        self.device = torch.device(device)
        bcmap = download_bcmap(grid)
        n = (grid.shape[2], grid.shape[1], grid.shape[0])
        self.plans = {r: SlabPlan(n, grid.NGHOSTS, bcmap, r, comm.world) for r in comm.ranks}
        self.ops = LibSlabOps(system, grid, self.plans, device)
        self.stepper = SlabStepper(self.plans, comm, self.ops)

    def local(self, r):
        """Rank r's Evolution (its slab, halo planes included)."""
        return self.ops.ev[r]

    def set_state(self, y):
        """Each local rank takes its window of the whole-grid state y
        (ngf, n2, n1, n0), on the host or any device."""
        for r, pl in self.plans.items():
            self.ops.ev[r].y_n.copy_(torch.as_tensor(y)[:, pl.w0:pl.w1])

    def owned_state(self, r):
        """(first global plane, rank r's owned planes of y_n)."""
        pl = self.plans[r]
        a, b = pl.owned_planes
        return pl.w0 + a, self.ops.ev[r].y_n[:, a:b]

    def step(self, dt):
        self.stepper.step(dt)

    def capture(self, dt, n_steps=1):
        """Captures n_steps slab steps of every local rank into one CUDA graph
        and returns a callable that replays them (LocalComm only: its
        exchanges are device copies on the capturing stream; NCCL exchanges
        between processes are not captured here).  The first step runs once
        outside the graph and is undone."""
        if not isinstance(self.comm, LocalComm):
            raise ValueError("capture needs the in-process communicator (LocalComm)")
        g = torch.cuda.CUDAGraph()
        snap = {r: ev.y_n.clone() for r, ev in self.ops.ev.items()}
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.step(dt)  # warm-up: module load, exchange buffers
        torch.cuda.current_stream(self.device).wait_stream(side)
        with torch.cuda.graph(g):
            for _ in range(n_steps):
                self.step(dt)
        for r, ev in self.ops.ev.items():
            ev.y_n.copy_(snap[r])
        for ev in self.ops.ev.values():
            ev._sync_stream()

        def replay():
            g.replay()
        replay.graph = g
        return replay

    def l2_norm(self, gf=0):
        """RMS over the whole grid's interior points of gridfunction gf of
        y_n: the ranks' sums of squares and point counts, all-reduced."""
        vals = {}
        for r in self.comm.ranks:
            ev = self.ops.ev[r]
            ev._sync_stream()
            scratch = torch.empty(1024, dtype=torch.float64, device=self.device)
            res = torch.empty(2, dtype=torch.float64, device=self.device)
            _lib.check(ev.lib.nrgpu_l2_norm_sq(C.byref(ev.grid.params), _lib.ptr(ev.y_n), gf, _lib.ptr(scratch),
                                               1024, _lib.ptr(res)), "nrgpu_l2_norm_sq")
            vals[r] = res
        tot = self.comm.allreduce_sum(vals)[self.comm.ranks[0]]
        s, n = tot.tolist()
        return (s / n) ** 0.5
