"""Continuous-batching server for shock-tube solves.

Requests (a tube's parameters and initial particles, with an end time) arrive
over time.  The server keeps every admitted tube's particle state resident on
the GPU and advances all of them together, one batch context, in epochs of
``epoch_steps`` steps (one CUDA graph replay per step).  Between epochs it
  * retires tubes that reached their end time (their state is downloaded and
    the request completes),
  * admits waiting requests while the estimated device memory of the batch
    stays within ``budget_bytes`` and the batch has fewer than ``max_tubes``
    tubes,
  * and, when the membership changed, rebuilds the batch: running tubes are
    carried into the new context device to device (``ds_copy_tube``), new ones
    are uploaded.
Each tube advances with its own CFL step and stops at its own end time, and
nothing in a tube's arithmetic depends on the other tubes of the batch, so a
request's result is the same alone and in the mix.
"""
from __future__ import annotations

import dataclasses
import time
from typing import Callable, List, Optional

import numpy as np

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


def memory_estimate(P: Params, species: List[Species]) -> int:
    n = sum(s.n for s in species)
    ncells, nidic = grid_sizes(P)
    ns = 1 + P.n_dust
    b = n * BYTES_PER_PARTICLE + ns * (ncells + 2) * BYTES_PER_KEY + ns * (nidic + 2) * BYTES_PER_IDIC_KEY
    if P.precision == "fp32" and P.force_list != -1:
        # recorded force neighbours: cap entries for every slot of the gas
        # chunks, a count per slot, a flag per chunk
        cap = P.force_list if P.force_list > 0 else 256
        chunks = -(-species[0].n // 128)
        b += chunks * 128 * 4 * cap + chunks + 4 * n
    return int(b)


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    params: Params
    species: List[Species]
    t_end: float

    @property
    def particles(self) -> int:
        return sum(s.n for s in self.species)


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
        self.particle_steps = 0

    def _params(self, r: Request) -> Params:
        P = r.params.copy()
        P.T_end = r.t_end
        P.precision = self.precision
        return P

    def estimate(self, r: Request) -> int:
        """Device bytes the request takes in this server's batch."""
        return memory_estimate(self._params(r), r.species)

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
                        sp = [S.get_species(t, s, template=r.species[s]) for s in range(1 + r.params.n_dust)]
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
                members = [r for _, r in keep] + joined
                if members:
                    N = Solver([self._params(r) for r in members])
                    for k, (t_old, r) in enumerate(keep):
                        N.copy_tube_from(k, S, t_old)
                    for k, r in enumerate(joined, start=len(keep)):
                        N.set_tube(k, r.species)
                    N.step(0)  # make the carried tubes resident before the old context goes
                else:
                    N = None
                if S is not None:
                    S.close()
                S = N
                active = members
                self.rebuilds += 1
            if S is None:
                continue
            S.step(self.epoch_steps)
            self.particle_steps += sum(r.particles for r in active) * self.epoch_steps
            if on_epoch:
                on_epoch(self, active)
        if S is not None:
            S.close()
        return sorted(results, key=lambda r: r.rid)


def poisson_requests(rate_per_s: float, n: int, seed: int, make_tube, t_end_range=(0.05, 0.2)) -> List[Request]:
    """n requests with exponential inter-arrival times (rate_per_s), seeded;
    make_tube(rng) -> (params, species)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate_per_s))
        P, sp = make_tube(rng)
        out.append(Request(i, t, P, sp, float(rng.uniform(*t_end_range))))
    return out


def run_alone(r: Request, precision: str = "fp32") -> List[Species]:
    """The same request solved on its own (for the alone-vs-mix check)."""
    P = r.params.copy()
    P.T_end = r.t_end
    P.precision = precision
    with Solver(P) as S:
        S.set_tube(0, r.species)
        while S.time(0)[0] < r.t_end:
            S.step(50)
        return [S.get_species(0, s, template=r.species[s]) for s in range(1 + P.n_dust)]
