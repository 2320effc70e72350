"""CPU oracle (test infrastructure only): jsolver's 1D grid restated.

Follows jsolver/grid_1d.py:82-112 (``compute_dependent_vars``, ``build_grid``). Only the
fields the solver reads (``mx``, ``idel``, ``is_linear``) and the cell centres used to
build manufactured problems are needed by the oracle.
"""
import numpy as np


class OracleGrid1D:
    def __init__(self, mx, xb=0.0, xe=1.0, rim=1, grid_type=0, centered=True):
        self.mx, self.xb, self.xe, self.rim = mx, xb, xe, rim
        self.grid_type, self.centered = grid_type, centered
        self.nx = mx + 1
        self.length = xe - xb
        self.del_ = self.length / (mx if centered else self.nx)
        self.idel = 1 / self.del_
        ipos = np.arange(-rim, mx + rim + 2)
        if grid_type == 0:
            self.edges = (ipos - 0.5 if centered else ipos) * self.del_ + xb
        elif grid_type == 1:
            self.edges = (ipos + 2 * np.sin(2 * np.pi * ipos / self.nx)) * self.del_ + xb
        else:
            raise ValueError("No such grid grid_type: {}".format(grid_type))
        self.centers = 0.5 * (self.edges[:-1] + self.edges[1:])
        self.widths = self.edges[1:] - self.edges[:-1]
        self.is_linear = grid_type == 0
