"""Continuous-batching server for shock-tube solves.

Requests (a tube's parameters and initial particles, or a generator that makes
them on the device, with an end time) arrive over time.  The server keeps every admitted tube's particle state resident on
the GPU and advances all of them together, one batch context, in epochs of
``epoch_steps`` steps (one CUDA graph replay per step).  Between epochs it
  * retires tubes that reached their end time (their state is downloaded and
    the request completes),
  * admits waiting requests while the estimated device memory of the batch
    stays within ``budget_bytes`` and the batch has fewer than ``max_tubes``
    tubes,
  * and, when the membership changed, rebuilds the batch: running tubes are
    carried into the new context device to device (``ds_copy_tube``), new ones
    are generated on the device (``ds_init_tube``) or uploaded.
Each tube advances with its own CFL step and stops at its own end time, and
nothing in a tube's arithmetic depends on the other tubes of the batch, so a
request's result is the same alone and in the mix.
"""
from __future__ import annotations

import dataclasses
import time
from typing import Callable, List, Optional, Sequence, Union

import numpy as np

from .ic import DeviceIC
from .params import Params
from .solver import Solver
from .species import Species

# device bytes per particle and per cell key of a batch context (ds_api.cu
# allocations): two copies of 15 FP64 fields and 2 ints, FP32 copies, scratch,
# the download staging (every field and Ind)
BYTES_PER_PARTICLE = 2 * (15 * 8 + 8) + 3 * 16 + 4 * 8 + 14 * 4 + (15 * 8 + 4)
BYTES_PER_KEY = 4 + 8 + 1
BYTES_PER_IDIC_KEY = 4 + 14 * 8 + 4


def grid_sizes(P: Params):
    """(neighbour cells, IDIC cells) of a tube, as the library derives them."""
    w = P.cell_width()
    cnx = int((P.X_max - P.X_min) / w)
    cny = int((P.Y_max - P.Y_min) / w)
    cnz = int((P.Z_max - P.Z_min) / w)
    if P.mode.grid_proper:
        ny = int((P.Y_max - P.Y_min) / w) if P.mode.periodic_y else cny + 1
        nz = int((P.Z_max - P.Z_min) / w) if P.mode.periodic_z else cnz + 1
        ncells = (cnx + 1) * max(ny, 1) * max(nz, 1)
    else:
        ncells = (cnx + 1) * (cny + 1) * (cnz + 1)
    aw = P.idic_width()
    nidic = (int((P.X_max - P.X_min) / aw) + 1) * (int((P.Y_max - P.Y_min) / aw) + 1) * \
        (int((P.Z_max - P.Z_min) / aw) + 1)
    return ncells, nidic


def memory_estimate(P: Params, species: Sequence[Union[Species, int]]) -> int:
    """Device bytes of one tube in a batch context; species: the species or
    their particle counts (gas first)."""
    counts = [s if isinstance(s, (int, np.integer)) else s.n for s in species]
    n = sum(counts)
    ncells, nidic = grid_sizes(P)
    ns = 1 + P.n_dust
    b = n * BYTES_PER_PARTICLE + ns * (ncells + 2) * BYTES_PER_KEY + ns * (nidic + 2) * BYTES_PER_IDIC_KEY
    if P.precision == "fp32" and P.force_list != -1:
        # recorded force neighbours: cap entries for every slot of the gas
        # chunks, a count per slot, a flag per chunk
        cap = P.force_list if P.force_list > 0 else 256
        chunks = -(-counts[0] // 128)
        b += chunks * 128 * 4 * cap + chunks + 4 * n
    return int(b)


@dataclasses.dataclass
class Request:
    """A tube to solve: its initial particles (species), or ic, a generator run
    on the device at admission (its plan gives params and the counts)."""
    rid: int
    arrival: float          # seconds after the start of the run
    params: Params
    species: Optional[List[Species]]
    t_end: float
    ic: Optional[DeviceIC] = None

    @property
    def counts(self) -> List[int]:
        if self.species is not None:
            return [s.n for s in self.species]
        if not hasattr(self, "_counts"):
            self._counts = self.ic.plan(self.params)[1]
        return self._counts

    @property
    def particles(self) -> int:
        return sum(self.counts)

    def put(self, S: Solver, tube: int):
        """Place the initial particles into tube `tube` of S."""
        if self.ic is not None:
            S.init_tube(tube, self.ic)
        else:
            S.set_tube(tube, self.species)


@dataclasses.dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    steps: int
    particles: int
    species: List[Species]

    @property
    def time_to_solution(self) -> float:
        return self.finished - self.arrival


class Server:
    def __init__(self, budget_bytes: float = 150e9, epoch_steps: int = 10, max_tubes: int = 64,
                 precision: str = "fp32", clock: Callable[[], float] = time.perf_counter):
        self.budget = budget_bytes
        self.epoch_steps = epoch_steps
        self.max_tubes = max_tubes
        self.precision = precision
        self.clock = clock
        self.rebuilds = 0
        self.rebuild_s = 0.0  # wall time spent rebuilding the batch (new context, carried and new tubes)
        self.particle_steps = 0

    def _params(self, r: Request) -> Params:
        P = r.params.copy()
        P.T_end = r.t_end
        P.precision = self.precision
        return P

    def estimate(self, r: Request) -> int:
        """Device bytes the request takes in this server's batch."""
        return memory_estimate(self._params(r), r.counts)

    def run(self, requests: List[Request], on_epoch: Optional[Callable] = None) -> List[Result]:
        pending = sorted(requests, key=lambda r: r.arrival)
        queue: List[Request] = []
        active: List[Request] = []       # in tube order of the current context
        admitted_at = {}
        results: List[Result] = []
        S: Optional[Solver] = None
        t0 = self.clock()
        while pending or queue or active:
            now = self.clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.pop(0))
            if not active and not queue:
                # idle until the next arrival
                wait = pending[0].arrival - now
                if wait > 0:
                    time.sleep(min(wait, 0.05))
                continue
            # retire finished tubes
            keep = []
            if S is not None:
                for t, r in enumerate(active):
                    Tm, _, nstep = S.time(t)
                    if Tm >= r.t_end:
                        sp = [S.get_species(t, s) for s in range(1 + r.params.n_dust)]
                        results.append(Result(r.rid, r.arrival, admitted_at[r.rid], self.clock() - t0, nstep,
                                              r.particles, sp))
                    else:
                        keep.append((t, r))
            # admit waiting requests within the memory budget
            used = sum(self.estimate(r) for _, r in keep)
            joined = []
            while queue and len(keep) + len(joined) < self.max_tubes:
                need = self.estimate(queue[0])
                if need > self.budget:
                    raise ValueError(f"request {queue[0].rid} needs ~{need} device bytes, more than the "
                                     f"budget of {self.budget:.0f}")
                if used + need > self.budget:
                    break
                r = queue.pop(0)
                used += need
                joined.append(r)
                admitted_at[r.rid] = self.clock() - t0
            if joined or len(keep) != len(active):
                rb0 = self.clock()
                members = [r for _, r in keep] + joined
                if members:
                    N = Solver([self._params(r) for r in members])
                    for k, (t_old, r) in enumerate(keep):
                        N.copy_tube_from(k, S, t_old)
                    for k, r in enumerate(joined, start=len(keep)):
                        r.put(N, k)
                    N.step(0)  # make the carried tubes resident before the old context goes
                else:
                    N = None
                if S is not None:
                    S.close()
                S = N
                active = members
                self.rebuilds += 1
                self.rebuild_s += self.clock() - rb0
            if S is None:
                continue
            S.step(self.epoch_steps)
            self.particle_steps += sum(r.particles for r in active) * self.epoch_steps
            if on_epoch:
                on_epoch(self, active)
        if S is not None:
            S.close()
        return sorted(results, key=lambda r: r.rid)


def one_at_a_time(requests: List[Request], precision: str, clock: Callable[[], float] = time.perf_counter,
                  group: int = 10) -> List[Result]:
    """The same requests solved one at a time, in arrival order, each in its own
    context (made, filled, stepped to its end time, read back, closed) as a
    plain single-tube host would; a request that arrives while another runs
    waits.  Measured in real time from the first arrival schedule, so the
    time to solution includes the queueing a one-at-a-time service causes."""
    results = []
    t0 = clock()
    for r in sorted(requests, key=lambda q: q.arrival):
        wait = r.arrival - (clock() - t0)
        if wait > 0:
            time.sleep(wait)
        start = clock() - t0
        P = r.params.copy()
        P.T_end = r.t_end
        P.precision = precision
        with Solver(P) as S:
            r.put(S, 0)
            while S.time(0)[0] < r.t_end:
                S.step(group)
            nstep = S.time(0)[2]
            sp = [S.get_species(0, s) for s in range(1 + P.n_dust)]
        results.append(Result(r.rid, r.arrival, start, clock() - t0, nstep, r.particles, sp))
    return sorted(results, key=lambda q: q.rid)


def poisson_requests(rate_per_s: float, n: int, seed: int, make_tube, t_end_range=(0.05, 0.2)) -> List[Request]:
    """n requests with exponential inter-arrival times (rate_per_s), seeded;
    make_tube(rng) -> (params, species) or (params, DeviceIC)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate_per_s))
        P, sp = make_tube(rng)
        t_end = float(rng.uniform(*t_end_range))
        if isinstance(sp, DeviceIC):
            out.append(Request(i, t, P, None, t_end, ic=sp))
        else:
            out.append(Request(i, t, P, sp, t_end))
    return out


def device_uneven_tube(rng):
    """(params, DeviceIC) of one tube of the uneven-batch distributions
    (ic.draw_tube_params), generated on the device at admission."""
    from .ic import draw_tube_params
    spec = DeviceIC.uneven(**draw_tube_params(rng))
    return spec.plan()[0], spec


def run_alone(r: Request, precision: str = "fp32") -> List[Species]:
    """The same request solved on its own (for the alone-vs-mix check)."""
    P = r.params.copy()
    P.T_end = r.t_end
    P.precision = precision
    with Solver(P) as S:
        r.put(S, 0)
        while S.time(0)[0] < r.t_end:
            S.step(50)
        return [S.get_species(0, s) for s in range(1 + P.n_dust)]
