"""One tube cut into x-slabs across processes (one process per GPU).

The reference runs one tube on one device (kernel.cu:1793).  A tube larger
than one GPU's share of a job is cut along x into slabs, one per rank:

* Ownership.  Rank r owns every particle (gas and dust) whose IDIC cell column
  lies in [K_r, K_{r+1}); the columns are computed as the step computes them
  (``solver.idic_columns``), so every IDIC cell -- whose sums, solve and
  relaxation couple the gas and dust in it (kernel.cu:2060-2437) -- lives in
  one slab with all its particles.  The column bounds balance the gas counts
  at the start and stay fixed; particles that cross a bound move to the other
  rank after the step.
* Ghosts.  Before the density, each rank receives the gas of other slabs
  within 2 h_max of its own gas (h_max: the largest h of the tube): the
  partners of its density and force sums.  They enter its local tube frozen
  (Ind = 1), so they are summed over but not updated, and their own density
  is not computed there.
* One step (the library's split step):
    ds_step_density    sort, density, EOS on every rank;
    allreduce(min)     of the CFL candidates (the only collective of the
                       step's arithmetic; none with a fixed step);
    halo exchange      the ghosts' density and pressure from their owners
                       (ds_set_gas_hydro), so the force sees the same values
                       as on one domain;
    ds_step_complete   t_stop, dt, force, IDIC cells, update.
  Then owned particles that left the slab's columns go to their new owner.
* Order.  A rank's local particles (owned and ghosts) are kept in global
  index order, so cells list them in the order one domain does: on the FP64
  path a slab run equals the single-domain run bit for bit.

Scope: the proper cell and IDIC grids, constant stopping times (the
reference's index coupling, IDIC.h:8 and IDIC.h:86, pairs particle i of the
gas with particle i of the dust, which a spatial cut separates), no per-step
dust density.

Exchanges use torch.distributed (gloo on CPU tensors, NCCL on CUDA tensors):
counts by all_gather, particles by point-to-point sends.  The local step runs
through a backend: ``SolverBackend`` (the CUDA library) here; the tests add
one over the CPU oracle.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np

from .params import Params
from .species import FLOAT_FIELDS, Species

GHOST_IND = 1  # frozen in the local tube: a partner in the sums, never updated
NCOL = len(FLOAT_FIELDS) + 2  # packed particle: the fields, Ind, global index


def check_supported(P: Params):
    m = P.mode
    why = []
    if not m.grid_proper:
        why.append("the proper cell grid (grid_proper)")
    if not m.idic_proper:
        why.append("the proper IDIC grid (idic_proper)")
    if not m.tstop_const:
        why.append("constant stopping times (tstop_const)")
    if m.ref_index_coupling:
        why.append("no index coupling (ref_index_coupling off)")
    if m.dust_rho:
        why.append("no per-step dust density (dust_rho off)")
    if why:
        raise ValueError("slab decomposition needs " + ", ".join(why))


def split_columns(cols: np.ndarray, nranks: int) -> np.ndarray:
    """Column bounds K[0..nranks] (K[0] = -inf, K[-1] = +inf as int bounds)
    that give every rank about the same number of the given columns' particles
    and at least one column each."""
    lo, hi = int(cols.min()), int(cols.max())
    counts = np.bincount(cols - lo, minlength=hi - lo + 1)
    cum = np.cumsum(counts)
    K = [np.iinfo(np.int32).min]
    for r in range(1, nranks):
        k = int(np.searchsorted(cum, cum[-1] * r / nranks)) + 1 + lo
        k = max(k, K[-1] + 1 if r > 1 else lo + 1)
        K.append(min(k, hi - (nranks - 1 - r)))
    K.append(np.iinfo(np.int32).max)
    return np.array(K, dtype=np.int64)


def pack(sp: Species, gid: np.ndarray, idx=None) -> np.ndarray:
    idx = np.arange(sp.n) if idx is None else idx
    out = np.empty((len(idx), NCOL), dtype=np.float64)
    for k, f in enumerate(FLOAT_FIELDS):
        out[:, k] = getattr(sp, f)[idx]
    out[:, -2] = sp.ind[idx]
    out[:, -1] = gid[idx]
    return out


def unpack(a: np.ndarray):
    kw = {f: np.ascontiguousarray(a[:, k]) for k, f in enumerate(FLOAT_FIELDS)}
    sp = Species(ind=np.ascontiguousarray(a[:, -2]).astype(np.int32), **kw)
    return sp, a[:, -1].astype(np.int64)


def concat(parts: Sequence[Species]) -> Species:
    kw = {f: np.concatenate([getattr(p, f) for p in parts]) for f in FLOAT_FIELDS}
    return Species(ind=np.concatenate([p.ind for p in parts]).astype(np.int32), **kw)


class TorchComm:
    """The exchanges over a torch.distributed process group."""

    def __init__(self, group=None, device=None):
        import torch
        import torch.distributed as dist
        self.torch, self.dist, self.group = torch, dist, group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)
        if device is None:
            nccl = dist.get_backend(group) == "nccl"
            device = torch.device("cuda", torch.cuda.current_device()) if nccl else torch.device("cpu")
        self.device = device

    def _global(self, r):
        return self.dist.get_global_rank(self.group, r) if self.group is not None else r

    def allreduce_min(self, v: float) -> float:
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MIN, group=self.group)
        return float(t.item())

    def allreduce_sum(self, v: np.ndarray) -> np.ndarray:
        t = self.torch.tensor(np.asarray(v, dtype=np.float64), device=self.device)
        self.dist.all_reduce(t, group=self.group)
        return t.cpu().numpy()

    def exchange(self, send: List[np.ndarray], ncol: int) -> List[np.ndarray]:
        """send[r]: rows (float64, ncol columns) for rank r; returns the rows
        every rank sent here, by source rank."""
        T, D = self.torch, self.dist
        counts = T.tensor([len(a) for a in send], dtype=T.int64, device=self.device)
        allc = [T.zeros(self.size, dtype=T.int64, device=self.device) for _ in range(self.size)]
        D.all_gather(allc, counts, group=self.group)
        reqs, bufs, outgoing = [], [None] * self.size, []
        for r in range(self.size):
            if r != self.rank and len(send[r]):
                t = T.from_numpy(np.ascontiguousarray(send[r], dtype=np.float64)).to(self.device)
                outgoing.append(t)  # alive until every send has completed
                reqs.append(D.isend(t, self._global(r), group=self.group))
        for r in range(self.size):
            n = int(allc[r][self.rank].item())
            if r != self.rank and n:
                bufs[r] = T.empty((n, ncol), dtype=T.float64, device=self.device)
                reqs.append(D.irecv(bufs[r], self._global(r), group=self.group))
        for q in reqs:
            q.wait()
        out = []
        for r in range(self.size):
            if r == self.rank:
                out.append(np.asarray(send[r], dtype=np.float64).reshape(-1, ncol))
            elif bufs[r] is None:
                out.append(np.zeros((0, ncol), dtype=np.float64))
            else:
                out.append(bufs[r].cpu().numpy())
        return out


class SlabTube:
    """This rank's slab of one tube.  Every rank passes the same parameters and
    the same initial particles (global index = position in those arrays)."""

    def __init__(self, P: Params, species: Sequence[Species], backend, comm):
        check_supported(P)
        self.P, self.backend, self.comm = P, backend, comm
        self.ns = 1 + P.n_dust
        sp = [s.copy().fill_missing() for s in species]
        g = sp[0]
        hmax = float(g.h.max()) if (P.mode.h_per_particle and g.n) else P.h
        # partners within 2 h_max; the margin covers the rounding of positions
        self.halo = 2.0 * hmax * (1.0 + 1e-6) + 1e-12 * max(abs(P.X_min), abs(P.X_max), 1.0)
        self.K = split_columns(backend.columns(g.x), comm.size)
        self.own, self.gid = [], []
        for s in range(self.ns):
            keep = self._mine(backend.columns(sp[s].x))
            idx = np.nonzero(keep)[0]
            self.own.append(sp[s].take(idx))
            self.gid.append(idx.astype(np.int64))
        self.steps = 0
        self.migrated = 0  # particles this rank received from other slabs after a step

    def _owner(self, cols):
        return np.searchsorted(self.K, cols, side="right") - 1

    def _mine(self, cols):
        return (cols >= self.K[self.comm.rank]) & (cols < self.K[self.comm.rank + 1])

    # -- one step -------------------------------------------------------------
    def step(self, n: int = 1):
        for _ in range(n):
            if self.backend.time()[0] >= self.P.T_end:
                continue
            self._step()

    def _step(self):
        C, B, me = self.comm, self.backend, self.comm.rank
        g, ggid = self.own[0], self.gid[0]
        # the gas x-range of every slab, then the gas each other slab needs
        lohi = np.array([g.x.min(), g.x.max()] if g.n else [np.inf, -np.inf])
        ranges = C.exchange([lohi.reshape(1, 2)] * C.size, 2)
        sent = []
        for r in range(C.size):
            if r == me or not len(ranges[r]):
                sent.append(np.zeros(0, dtype=np.int64))
                continue
            lo, hi = ranges[r][0]
            sent.append(np.nonzero((g.x >= lo - self.halo) & (g.x <= hi + self.halo))[0])
        recv = C.exchange([pack(g, ggid, sent[r]) if r != me else np.zeros((0, NCOL)) for r in range(C.size)], NCOL)
        ghosts = [unpack(recv[r]) for r in range(C.size) if r != me and len(recv[r])]
        src = np.concatenate([np.full(len(recv[r]), r) for r in range(C.size) if r != me and len(recv[r])]
                             + [np.zeros(0, dtype=np.int64)])
        # the local gas in global index order; ghosts frozen
        parts = [g] + [s for s, _ in ghosts]
        gids = np.concatenate([ggid] + [i for _, i in ghosts])
        is_ghost = np.concatenate([np.zeros(g.n, bool)] + [np.ones(s.n, bool) for s, _ in ghosts])
        lg = concat(parts)
        lg.ind = np.where(is_ghost, GHOST_IND, lg.ind).astype(np.int32)
        order = np.argsort(gids, kind="stable")
        lg = lg.take(order)
        is_ghost = is_ghost[order]
        pos = np.empty(len(order), dtype=np.int64)
        pos[order] = np.arange(len(order))  # local index of each (owned, then received) gas particle
        ghost_local = pos[g.n:]              # by source rank, in the order each source sent them
        B.load([lg] + [self.own[s] for s in range(1, self.ns)])
        B.density()
        if self.P.mode.cfl:
            B.set_cfl_min(C.allreduce_min(B.cfl_min()))
        # the ghosts' density and pressure, as their owners computed them
        rho_p = B.gas_rho_p()
        own_local = pos[:g.n]
        hy = [np.stack([rho_p[0][own_local[sent[r]]], rho_p[1][own_local[sent[r]]]], 1) if r != me
              else np.zeros((0, 2)) for r in range(C.size)]
        back = C.exchange(hy, 2)
        vals = np.concatenate([back[r] for r in range(C.size) if r != me and len(back[r])] + [np.zeros((0, 2))])
        assert len(vals) == len(ghost_local) and (np.sort(src) == src).all()
        B.set_gas_hydro(ghost_local.astype(np.int32), vals[:, 0], vals[:, 1])
        B.complete()
        out = B.fetch()
        # owned particles, then those that left the slab to their new owners
        new_own, new_gid = [], []
        for s in range(self.ns):
            if s == 0:
                keep = np.nonzero(~is_ghost)[0]
                sp, gid = out[0].take(keep), np.sort(gids)[keep]
            else:
                sp, gid = out[s], self.gid[s]
            cols = B.columns(sp.x)
            dst = self._owner(cols)
            stay = dst == me
            mig = C.exchange([pack(sp, gid, np.nonzero(dst == r)[0]) if r != me else np.zeros((0, NCOL))
                              for r in range(C.size)], NCOL)
            got = [unpack(mig[r]) for r in range(C.size) if r != me and len(mig[r])]
            self.migrated += sum(len(i) for _, i in got)
            allsp = concat([sp.take(np.nonzero(stay)[0])] + [x for x, _ in got])
            allg = np.concatenate([gid[stay]] + [i for _, i in got])
            o = np.argsort(allg, kind="stable")
            new_own.append(allsp.take(o))
            new_gid.append(allg[o])
        self.own, self.gid = new_own, new_gid
        self.steps += 1

    # -- results --------------------------------------------------------------
    def time(self):
        return self.backend.time()

    def gather(self, s: int, n_total: int) -> Species:
        """Species s of the whole tube in global index order (every rank)."""
        rows = self.comm.exchange([pack(self.own[s], self.gid[s])] * self.comm.size, NCOL)
        sp, gid = unpack(np.concatenate(rows))
        assert len(gid) == n_total and (np.sort(gid) == np.arange(n_total)).all(), "particles lost or duplicated"
        return sp.take(np.argsort(gid))

    def conservation(self) -> np.ndarray:
        """Mass, momentum (x, y, z) and kinetic + internal energy of the whole
        tube: FP64 sums per rank, then an allreduce(sum)."""
        tot = np.zeros(5)
        for s in range(self.ns):
            sp = self.own[s]
            tot[0] += sp.m.sum()
            tot[1] += (sp.m * sp.vx).sum()
            tot[2] += (sp.m * sp.vy).sum()
            tot[3] += (sp.m * sp.vz).sum()
            tot[4] += (0.5 * sp.m * (sp.vx ** 2 + sp.vy ** 2 + sp.vz ** 2)).sum() + (sp.m * sp.e).sum() * (s == 0)
        return self.comm.allreduce_sum(tot)


class SolverBackend:
    """The local step on this process's GPU through the C ABI.  A slab's
    particle counts change from step to step while a context's are fixed, so
    the context holds a capacity per species; the unused slots hold parked
    particles -- frozen, massless, past the tube's x end beyond any real
    particle's cells -- in an x extension of the box that leaves every real
    particle's cells, IDIC cells and partners as they are."""

    def __init__(self, P: Params, slack: float = 1.25, seed: int = 0):
        from .solver import idic_columns
        self._cols = idic_columns
        self.P = P.copy()
        w = max(P.cell_width(), P.h) + P.list_skin * P.h
        self.park_x = P.X_max + (2 * P.stencil + 4) * w + 2 * P.h
        self.Pext = P.copy()
        self.Pext.X_max = self.park_x + 4 * w
        self.slack, self.rng = slack, np.random.default_rng(seed)
        self.S, self.cap, self.n = None, None, None
        self.Tm, self.nstep = 0.0, 0

    def columns(self, x):
        return self._cols(self.P, x).astype(np.int64)

    def _park(self, n):
        P = self.P
        kw = {f: np.zeros(n) for f in FLOAT_FIELDS}
        kw["x"] = self.park_x + self.rng.random(n) * 2.0 * max(P.cell_width(), P.h)
        kw["y"] = P.Y_min + self.rng.random(n) * (P.Y_max - P.Y_min)
        kw["z"] = P.Z_min + self.rng.random(n) * (P.Z_max - P.Z_min)
        kw["rho"][:] = 1.0
        kw["p"][:] = 1.0
        kw["e"][:] = 1.0
        kw["h"][:] = P.h
        kw["ts"][:] = P.t_stop_const[0] if P.t_stop_const else 1.0
        return Species(ind=np.full(n, GHOST_IND, np.int32), **kw)

    def load(self, species: Sequence[Species]):
        from .solver import Solver
        counts = [s.n for s in species]
        if self.S is None or any(c > k for c, k in zip(counts, self.cap)):
            if self.S is not None:
                self.Tm, _, self.nstep = self.S.time(0)
                self.S.close()
            self.cap = [int(c * self.slack) + 64 for c in counts]
            # the reference's per-species particle limit (kernel.cu:1751) covers the capacity
            self.Pext.Maximum_particle = max(int(self.P.Maximum_particle), max(self.cap))
            self.S = Solver(self.Pext)
            self.S.set_time(0, self.Tm, self.nstep)
        self.S.set_tube(0, [concat([s, self._park(k - s.n)]) for s, k in zip(species, self.cap)])
        self.n = counts

    def density(self):
        self.S.step_density()

    def cfl_min(self) -> float:
        return self.S.cfl_min(0)

    def set_cfl_min(self, v: float):
        self.S.set_cfl_min(0, v)

    def gas_rho_p(self):
        g = self.S.get_species(0, 0)
        return g.rho[: self.n[0]], g.p[: self.n[0]]

    def set_gas_hydro(self, idx, rho, p):
        self.S.set_gas_hydro(0, idx, rho, p)

    def complete(self):
        self.S.step_complete()

    def fetch(self) -> List[Species]:
        return [self.S.get_species(0, s).take(np.arange(n)) for s, n in enumerate(self.n)]

    def time(self):
        if self.S is None:
            return self.Tm, self.nstep
        Tm, _, ns = self.S.time(0)
        return Tm, ns

    def close(self):
        if self.S is not None:
            self.S.close()
            self.S = None
