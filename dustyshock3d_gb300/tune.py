"""Autotuner for the FP32 neighbour sweeps of a batch of tubes.

Knobs (all results stay within the FP32 path's tolerance; none changes the
physics):
  * cell size and stencil: cells of width ~2 h_max searched 1 cell on each
    side, ~h_max searched up to 2, ~2/3 h_max up to 3 or ~h_max / 2 up to 4
    (each cell walks only as many as its particles' cut-offs reach; smaller
    cells screen fewer candidates per pair, in more rows);
  * list depth: candidate-list entries per thread (32 or 64), i.e. how many
    screened neighbours a thread stages before the pair work runs;
  * persistent sweeps: one block per chunk of 128 particles, or a grid of as
    many blocks as fit on the GPU at once, each claiming its next chunk;
  * threads per IDIC cell in the cell sums (2, 4 or 8);
  * reuse of the recorded neighbour lists across steps, with a skin of 0.1 or
    0.15 h_max (or none): a tube keeps its lists while its particles have not
    moved far enough relative to each other, and streams them instead of
    walking its cells.

The tuner times a few steps of each candidate on a sample of the batch (the
first ``sample`` tubes) with CUDA events and returns the fastest: first over
(stencil, cell width, list depth), then, for the winner, over (persistent,
threads per IDIC cell), then over the skins.  A skin pays off over a window of
steps (a rebuild every few steps), so that last stage times the winner with
and without each skin over ``skin_steps`` steps.
"""
from __future__ import annotations

import dataclasses
from typing import List, Sequence, Tuple, Union

from .ic import DeviceIC
from .params import Params
from .solver import Solver
from .species import Species

# (stencil, cell width / h_max, list depth)
CANDIDATES = [
    (2, 1.001, 32),
    (2, 1.001, 64),
    (1, 2.002, 32),
    (3, 0.6673, 32),
    (4, 0.5005, 32),
]
# (persistent sweeps, threads per IDIC cell), tried for the best of CANDIDATES
LAUNCH_CANDIDATES = [(0, 4), (1, 4), (0, 2), (0, 8), (1, 2), (1, 8)]
# list-reuse skins (units of the tube's h_max), tried last against no reuse
SKIN_CANDIDATES = (0.1, 0.15)


@dataclasses.dataclass
class Choice:
    stencil: int
    cell_factor: float
    list_depth: int
    ms_per_step: float
    persistent: int = 0
    idic_lanes: int = 4
    list_skin: float = 0.0


def apply(P: Params, stencil: int, cell_factor: float, list_depth: int, persistent: int = 0,
          idic_lanes: int = 4, list_skin: float = 0.0) -> Params:
    Q = P.copy()
    Q.stencil = stencil
    Q.cell_w = cell_factor * Q.h  # Q.h is the tube's largest smoothing length
    Q.list_depth = list_depth
    Q.persistent = persistent
    Q.idic_lanes = idic_lanes
    Q.list_skin = list_skin
    return Q


def _fits(P: Params) -> bool:
    """Periodic axes need 2*stencil+1 cells."""
    w = P.cell_width()
    need = 2 * P.stencil + 1
    if P.mode.periodic_y and int((P.Y_max - P.Y_min) / w) < need:
        return False
    if P.mode.periodic_z and int((P.Z_max - P.Z_min) / w) < need:
        return False
    return True


def put_tube(S: Solver, t: int, src) -> None:
    """Tube t of S from host particles (a species list) or from a generator run
    on the device (an ic.DeviceIC)."""
    if isinstance(src, DeviceIC):
        S.init_tube(t, src)
    else:
        S.set_tube(t, src)


def _time(sub, ps, warmup, steps) -> float:
    with Solver(ps) as S:
        for t, (_, sp) in enumerate(sub):
            put_tube(S, t, sp)
        S.step(warmup)
        return S.step_timed_graph(steps) / steps  # as ds_step runs the batch: its captured graphs


def tune(tubes: Sequence[Tuple[Params, Union[List[Species], DeviceIC]]], sample: int = 8, warmup: int = 2,
         steps: int = 3, precision: str = "fp32", candidates=CANDIDATES,
         launch_candidates=LAUNCH_CANDIDATES, skin_candidates=SKIN_CANDIDATES,
         skin_steps: int = 12) -> Tuple[Choice, list]:
    """tubes: (params, particles) pairs, the particles a species list or a
    DeviceIC generator.  The log holds (stencil, cell factor, list depth,
    persistent, threads per IDIC cell, skin, ms per step or None when the grid
    does not fit); the skin stage's rows (the winner without a skin among
    them) are timed over skin_steps steps."""
    sub = list(tubes[:sample])
    log = []
    best = None
    for stencil, factor, depth in candidates:
        ps = [apply(P, stencil, factor, depth) for P, _ in sub]
        for q in ps:
            q.precision = precision
        if not all(_fits(q) for q in ps):
            log.append((stencil, factor, depth, 0, 4, 0.0, None))
            continue
        ms = _time(sub, ps, warmup, steps)
        log.append((stencil, factor, depth, 0, 4, 0.0, ms))
        if best is None or ms < best.ms_per_step:
            best = Choice(stencil, factor, depth, ms)
    if best is None or precision != "fp32":
        return best, log
    for persistent, lanes in launch_candidates:
        if (persistent, lanes) == (0, 4):
            continue  # timed above
        ps = [apply(P, best.stencil, best.cell_factor, best.list_depth, persistent, lanes) for P, _ in sub]
        for q in ps:
            q.precision = precision
        ms = _time(sub, ps, warmup, steps)
        log.append((best.stencil, best.cell_factor, best.list_depth, persistent, lanes, 0.0, ms))
        if ms < best.ms_per_step:
            best = Choice(best.stencil, best.cell_factor, best.list_depth, ms, persistent, lanes)
    if not skin_candidates:
        return best, log
    win = None
    for skin in (0.0,) + tuple(skin_candidates):
        ps = [apply(P, best.stencil, best.cell_factor, best.list_depth, best.persistent, best.idic_lanes, skin)
              for P, _ in sub]
        for q in ps:
            q.precision = precision
        ms = _time(sub, ps, warmup, skin_steps)
        log.append((best.stencil, best.cell_factor, best.list_depth, best.persistent, best.idic_lanes, skin, ms))
        if win is None or ms < win.ms_per_step:
            win = dataclasses.replace(best, ms_per_step=ms, list_skin=skin)
    return win, log
