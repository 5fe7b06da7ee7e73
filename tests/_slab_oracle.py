"""The slab decomposition's local step on the CPU oracle (test infrastructure):
the backend protocol of dustyshock3d_gb300.slab over oracle.c's split step
(orc_step_density / orc_step_complete)."""
import ctypes

import numpy as np

from dustyshock3d_gb300.solver import idic_columns
from oracle.oracle import OracleState, lib


class OracleBackend:
    def __init__(self, P):
        assert P.precision == "fp64"
        self.P = P
        self.O = None
        self.Tm, self.nstep, self.dtmin = 0.0, 0, float("inf")

    def columns(self, x):
        return idic_columns(self.P, x).astype(np.int64)  # the FP64 path's columns = the oracle's

    def load(self, species):
        self.O = OracleState(self.P, species)
        self.O.Tm = self.Tm

    def density(self):
        d = ctypes.c_double(0.0)
        st = lib().orc_step_density(ctypes.byref(self.O.P), self.O._arr, ctypes.byref(d))
        assert st >= 0 and not (st & 9), st
        self.dtmin = d.value

    def cfl_min(self):
        return self.dtmin

    def set_cfl_min(self, v):
        self.dtmin = v

    def gas_rho_p(self):
        g = self.O.species[0]
        return g.rho.copy(), g.p.copy()

    def set_gas_hydro(self, idx, rho, p):
        g = self.O.species[0]  # the arrays oracle.c reads
        g.rho[idx] = rho
        g.p[idx] = p

    def complete(self):
        Tm, dt = ctypes.c_double(self.Tm), ctypes.c_double(0.0)
        st = lib().orc_step_complete(ctypes.byref(self.O.P), self.O._arr, ctypes.byref(Tm), self.dtmin,
                                     ctypes.byref(dt))
        assert st >= 0 and not (st & 9), st
        self.Tm = Tm.value
        self.nstep += 1

    def fetch(self):
        return [s.copy() for s in self.O.species]

    def time(self):
        return self.Tm, self.nstep
