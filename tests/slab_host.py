"""Host (CPU) per-rank operations for the slab-decomposed RK4 step, for the
gloo tests of nrpytutorial_gb300.slab: the same interface as LibSlabOps,
with the oracle's RHS (oracle/wave_maxwell.py) and numpy boundary rules in
the arithmetic of oracle/bcs.py.  Test infrastructure only."""
import numpy as np
import torch

import oracle.bcs as ob


def oracle_bcmap(gp):
    """The oracle's boundary map (oracle/bcs.py build_bcstruct) in the form
    of Evolution.bc_map(): parity bit t set where parity type t is -1."""
    layers = ob.build_bcstruct(gp)
    od, os_, idst, isrc, ipar = [], [], [], [], []
    num_ob, num_ib, dir_start, ib_start = [], [], [], []
    for outer_dirs, (d, s, p) in layers:
        starts = [len(od)]
        for arr in outer_dirs:
            od.extend(arr[:, 0].tolist())
            os_.extend(arr[:, 1].tolist())
            starts.append(len(od))
        dir_start.append(starts)
        num_ob.append(starts[-1] - starts[0])
        ib_start.append(len(idst))
        num_ib.append(len(d))
        idst.extend(d.tolist())
        isrc.extend(s.tolist())
        bits = (p < 0).astype(np.int64) << np.arange(10)
        ipar.extend(bits.sum(axis=1).tolist() if len(d) else [])
    a = lambda v: np.array(v, dtype=np.int64)
    return dict(outer_dest=a(od), outer_step=a(os_), inner_dest=a(idst), inner_src=a(isrc), inner_parity=a(ipar),
                num_ob=num_ob, num_ib=num_ib, ob_dir_start=dir_start, ib_start=ib_start)


class HostSlabOps:
    def __init__(self, gp, rhs_fn, parity_types, plans, y_global):
        self.gp = gp
        self.rhs_fn = rhs_fn
        self.ptypes = list(parity_types)
        self.ngf = len(self.ptypes)
        self.plans = plans
        n0, n1, n2 = plans[next(iter(plans))].n
        self.plane_points = n0 * n1
        self.buf = {}
        for r, pl in plans.items():
            shape = (self.ngf, pl.n2l, n1, n0)
            b = {k: torch.zeros(shape, dtype=torch.float64) for k in ("y_n", "rt", "k_odd", "k_even")}
            b["y_n"].copy_(torch.as_tensor(y_global[:, pl.w0:pl.w1]))
            self.buf[r] = b

    def stage_buffer(self, r, s):
        b = self.buf[r]
        return b["y_n"] if s == 3 else (b["k_odd"] if s % 2 == 0 else b["k_even"])

    def planes(self, r, s, a, b):
        return self.stage_buffer(r, s)[:, a:b]

    def new_buffer(self, r, n):
        return torch.empty(int(n), dtype=torch.float64)

    def substep(self, r, s, dt):
        pl = self.plans[r]
        b = {k: v.numpy() for k, v in self.buf[r].items()}
        inp = b["y_n"] if s == 0 else (b["k_odd"] if s % 2 == 1 else b["k_even"])
        full = np.zeros((self.ngf,) + self.gp.shape)
        full[:, pl.w0:pl.w1] = inp
        k = self.rhs_fn(full)[:, pl.w0:pl.w1]
        g = pl.ng
        I = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
        k = k[I]
        # the update expressions of oracle/bcs.py rk4_step, at interior points
        if s == 0:
            b["rt"][I] = k * dt * (1.0 / 6.0)
            b["k_odd"][I] = b["y_n"][I] + k * dt * (1.0 / 2.0)
        elif s == 1:
            b["rt"][I] = b["rt"][I] + k * dt * (1.0 / 3.0)
            b["k_even"][I] = b["y_n"][I] + k * dt * (1.0 / 2.0)
        elif s == 2:
            b["rt"][I] = b["rt"][I] + k * dt * (1.0 / 3.0)
            b["k_odd"][I] = b["y_n"][I] + k * dt
        else:
            b["y_n"][I] = b["y_n"][I] + b["rt"][I] + k * dt * (1.0 / 6.0)

    def outer(self, r, s, k):
        f = self.stage_buffer(r, s).numpy().reshape(self.ngf, -1)
        for d, st in self.plans[r].outer[k]:
            d, st = d.astype(np.int64), st.astype(np.int64)
            f[:, d] = 3.0 * f[:, d + st] - 3.0 * f[:, d + 2 * st] + 1.0 * f[:, d + 3 * st]

    def gather(self, r, s, k, q, out):
        idx = self.plans[r].inner_send[k][q].astype(np.int64)
        f = self.stage_buffer(r, s).numpy().reshape(self.ngf, -1)
        out.numpy()[:] = f[:, idx].T.reshape(-1)

    def scatter(self, r, s, k, recv):
        pl = self.plans[r]
        dest = pl.inner_dest[k].astype(np.int64)
        if len(dest) == 0:
            return
        bits = pl.inner_parity[k].astype(np.int64)
        vals = recv.numpy().reshape(len(dest), self.ngf)
        f = self.stage_buffer(r, s).numpy().reshape(self.ngf, -1)
        for g in range(self.ngf):
            sign = np.where((bits >> self.ptypes[g]) & 1, -1.0, 1.0)
            f[g, dest] = sign * vals[:, g]

    def post(self, r, s):
        pass
