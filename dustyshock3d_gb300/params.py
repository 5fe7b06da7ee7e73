"""Run parameters: the reference's Init.txt plus the extensions of this library.

The first 17 values mirror Init.txt, read positionally exactly as the
reference's ``main`` reads them (kernel.cu:1705-1723: one ``fgets`` per line,
the leading number parsed by ``sscanf`` and any trailing comment ignored; the
first line is a title).  Constants the reference hard-codes are fields here
with the reference's values: ``Gam_g`` = 1.4 (data.h:7) and
``Speed_of_sound_gas`` = 1.0 (kernel.cu:1744).

Extensions (no reference counterpart; the reference ignores extra lines, so an
extended Init.txt still runs the reference) are appended as ``name = value``
lines after line 18.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import List

MAX_DUST = 4


@dataclass
class Mode:
    """Behaviour switches.  ``Mode.reference()`` is the reference's own step."""

    periodic_y: bool = False
    periodic_z: bool = False
    h_per_particle: bool = False      # h_i per particle, symmetrised kernel gradient
    tstop_const: bool = False         # constant stopping time per species
    gas_accel_particle: bool = False  # gas relax uses its own A_i instead of the cell mean Psi
    ref_index_coupling: bool = True   # dust rho zeroed by gas Ind at the same index (IDIC.h:8)
    ref_eps_guard: bool = True        # every eps guard tests species 1's count (kernel.cu:2203)
    ref_solve2: bool = True           # two-species solve in the reference's operation order
    cfl: bool = False                 # CFL step instead of fixed tau
    dust_rho: bool = True             # dust self-density every step (kernel.cu:2029-2043)
    grid_proper: bool = False         # neighbour-cell stride nx instead of the aliasing Cnx
    idic_proper: bool = False         # IDIC-cell stride nx instead of the aliasing Nax

    @staticmethod
    def reference() -> "Mode":
        return Mode()

    @staticmethod
    def baseline() -> "Mode":
        """The shock-tube physics of the benchmark configurations."""
        return Mode(periodic_y=True, periodic_z=True, h_per_particle=True, tstop_const=True,
                    gas_accel_particle=True, ref_index_coupling=False, ref_eps_guard=False,
                    ref_solve2=False, cfl=True, dust_rho=False, grid_proper=True, idic_proper=True)

    def bits(self) -> int:
        b = 0
        for i, f in enumerate(dataclasses.fields(self)):
            if getattr(self, f.name):
                b |= 1 << i
        return b


# bit positions of Mode fields in the C-ABI flag word (same order as above)
MODE_BITS = {f.name: 1 << i for i, f in enumerate(dataclasses.fields(Mode))}


@dataclass
class Params:
    # Init.txt lines 2-18 (kernel.cu:1707-1723)
    X_min: float = -2.0
    X_max: float = 2.0
    Y_min: float = -2.0
    Y_max: float = 2.0
    Z_min: float = -2.0
    Z_max: float = 2.0
    Type_of_state: int = 0
    Maximum_particle: int = 1000000
    Particle_on_length: float = 40.0
    h: float = 0.1
    Coeff_h_dust_cell: float = 0.5
    tau: float = 5.0e-3
    T_end: float = 0.2
    T_out: float = 0.1
    alpha: float = 1.0
    beta: float = 2.0
    eps: float = 0.01
    # constants the reference hard-codes
    Gam_g: float = 1.4
    Speed_of_sound_gas: float = 1.0
    # extensions
    n_dust: int = 2
    mass_ratio: List[float] = field(default_factory=lambda: [0.75, 0.5])  # kernel.cu:1499-1502
    R_dust: List[float] = field(default_factory=lambda: [0.01, 1.0])
    t_stop_const: List[float] = field(default_factory=lambda: [1e-3, 1e-3])
    eps_empty: List[float] = field(default_factory=lambda: [0.5, 0.33])   # kernel.cu:2200, 2209
    t_empty: float = 1.0                                                   # kernel.cu:2160, 2188
    cell_w: float = 0.0   # neighbour cell width; 0 -> 2h (kernel.cu:1773)
    idic_w: float = 0.0   # IDIC cell width; 0 -> Coeff_h_dust_cell * h (kernel.cu:1577)
    cfl: float = 0.3
    stencil: int = 1      # cells searched on each side: 1 (the reference's 27 cells) or 2 (125 cells)
    list_depth: int = 0   # FP32 sweeps: candidate-list entries per thread (0 -> 32; 64)
    force_list: int = 0   # FP32: recorded force neighbours per gas particle (0 -> 256; -1 -> off)
    list_skin: float = 0.0  # FP32 with force lists: reuse the lists across steps, skin in units of h (0 -> off)
    persistent: int = 0   # FP32: neighbour sweeps on a persistent grid claiming chunks (1) or a block per chunk (0)
    idic_lanes: int = 0   # FP32: threads per IDIC cell in its cell sums, 2, 4 or 8 (0 -> 4)
    precision: str = "fp64"  # "fp64" or "fp32" (FP32 neighbour sums, FP64 state/IDIC)
    mode: Mode = field(default_factory=Mode)

    def cell_width(self) -> float:
        return self.cell_w if self.cell_w > 0 else 2.0 * self.h

    def idic_width(self) -> float:
        return self.idic_w if self.idic_w > 0 else self.Coeff_h_dust_cell * self.h

    def copy(self) -> "Params":
        c = dataclasses.replace(self)
        c.mass_ratio = list(self.mass_ratio)
        c.R_dust = list(self.R_dust)
        c.t_stop_const = list(self.t_stop_const)
        c.eps_empty = list(self.eps_empty)
        c.mode = dataclasses.replace(self.mode)
        return c


_INIT_ORDER = [
    ("X_min", float), ("X_max", float), ("Y_min", float), ("Y_max", float),
    ("Z_min", float), ("Z_max", float), ("Type_of_state", int), ("Maximum_particle", int),
    ("Particle_on_length", float), ("h", float), ("Coeff_h_dust_cell", float), ("tau", float),
    ("T_end", float), ("T_out", float), ("alpha", float), ("beta", float), ("eps", float),
]


# extension names that take one number (the Init.txt fields may be set by name too)
_FLOAT_FIELDS = {name for name, _ in _INIT_ORDER} | {"Gam_g", "Speed_of_sound_gas", "t_empty", "cell_w", "idic_w",
                                                      "cfl", "list_skin"}


def _leading_number(line: str, kind):
    """sscanf("%lf") / sscanf("%d") on one line: the leading number, rest ignored."""
    s = line.strip()
    end = 0
    allowed = "+-0123456789.eE" if kind is float else "+-0123456789"
    while end < len(s) and s[end] in allowed:
        end += 1
    tok = s[:end]
    while tok:
        try:
            return kind(tok)
        except ValueError:
            tok = tok[:-1]
    raise ValueError(f"no number at the start of {line!r}")


def parse_init_txt(text: str) -> Params:
    """Parse an Init.txt (kernel.cu:1705-1723) plus appended ``name = value`` lines."""
    lines = text.splitlines()
    if len(lines) < 18:
        raise ValueError(f"Init.txt needs a title line and 17 value lines, got {len(lines)} lines")
    P = Params()
    for (name, kind), line in zip(_INIT_ORDER, lines[1:18]):
        setattr(P, name, _leading_number(line, kind))
    for line in lines[18:]:
        body = line.split("//", 1)[0].strip()
        if not body or "=" not in body:
            continue
        key, val = (t.strip() for t in body.split("=", 1))
        if key == "ic" or key.startswith("ic."):
            continue  # initial conditions: ic.parse_ic_init_txt
        if key.startswith("mode."):
            if key[5:] not in MODE_BITS:
                raise ValueError(f"unknown mode switch {key!r}")
            setattr(P.mode, key[5:], val.lower() in ("1", "true", "yes", "on"))
        elif key in ("mass_ratio", "R_dust", "t_stop_const", "eps_empty"):
            setattr(P, key, [float(v) for v in val.replace(",", " ").split()])
        elif key in ("n_dust", "stencil", "list_depth", "force_list", "persistent", "idic_lanes"):
            setattr(P, key, int(val))
        elif key == "precision":
            P.precision = val
        elif key in _FLOAT_FIELDS:
            setattr(P, key, float(val))
        else:
            raise ValueError(f"unknown Init.txt extension {key!r}")
    return P


def read_init_txt(path: str) -> Params:
    with open(path, "r", encoding="latin-1") as f:
        return parse_init_txt(f.read())


def write_init_txt(P: Params, extensions: bool = True) -> str:
    out = ["// Initial parameters"]
    for name, kind in _INIT_ORDER:
        v = getattr(P, name)
        out.append(f"{v!r}\t\t// {name}" if kind is float else f"{int(v)}\t\t// {name}")
    if extensions:
        for k in ("Gam_g", "Speed_of_sound_gas", "t_empty", "cell_w", "idic_w", "cfl", "list_skin"):
            out.append(f"{k} = {getattr(P, k)!r}")
        out.append(f"n_dust = {P.n_dust}")
        out.append(f"stencil = {P.stencil}")
        out.append(f"list_depth = {P.list_depth}")
        out.append(f"force_list = {P.force_list}")
        out.append(f"persistent = {P.persistent}")
        out.append(f"idic_lanes = {P.idic_lanes}")
        for k in ("mass_ratio", "R_dust", "t_stop_const", "eps_empty"):
            out.append(f"{k} = " + " ".join(repr(float(v)) for v in getattr(P, k)))
        out.append(f"precision = {P.precision}")
        for f in dataclasses.fields(P.mode):
            out.append(f"mode.{f.name} = {int(getattr(P.mode, f.name))}")
    return "\n".join(out) + "\n"
