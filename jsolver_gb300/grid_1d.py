"""One-dimensional grid (geometry input of the solver).

Same fields, values and errors as davef96/jsolver's ``grid_1D`` (jsolver/grid_1d.py:4-113):
``mx``, ``nx = mx + 1``, ``centered``, ``rim``, ``xb``, ``xe``, ``grid_type``, ``length``,
``del_``, ``idel``, ``is_linear`` and the ``edges`` / ``centers`` / ``widths`` arrays;
equality and hashing on ``(mx, centered, grid_type, rim, xb, xe)``. It is a plain,
immutable-by-convention host object: the solver reads ``mx``, ``idel`` and ``is_linear``.
"""
import numpy as np


class grid_1D:  # noqa: N801  (reference class name)
    def __init__(self, mx, xb=0.0, xe=1.0, rim=1, grid_type=0, centered=True):
        self.centered = centered
        self.mx = mx
        self.rim = rim
        self.xb = xb
        self.xe = xe
        self.grid_type = grid_type
        self.compute_dependent_vars()
        self.build_grid()

    def __hash__(self):
        return hash((self.mx, self.centered, self.grid_type, self.rim, self.xb, self.xe))

    def __eq__(self, other):
        return isinstance(other, grid_1D) and (self.mx, self.centered, self.grid_type, self.rim, self.xb, self.xe) == (
            other.mx, other.centered, other.grid_type, other.rim, other.xb, other.xe)

    def compute_dependent_vars(self):
        """nx, length, cell width and its reciprocal (grid_1d.py:82-89)."""
        self.nx = self.mx + 1
        self.length = self.xe - self.xb
        self.del_ = self.length / (self.mx if self.centered else self.nx)
        self.idel = 1 / self.del_

    def build_grid(self):
        """Edges, centres and widths of the mx + 2 rim + 1 cells (grid_1d.py:91-112)."""
        ipos = np.arange(-self.rim, self.mx + self.rim + 2)
        if self.grid_type == 0:
            self.edges = (ipos - 0.5 if self.centered else ipos) * self.del_ + self.xb
        elif self.grid_type == 1:
            self.edges = (ipos + 2 * np.sin(2 * np.pi * ipos / self.nx)) * self.del_ + self.xb
        else:
            raise ValueError("No such grid grid_type: {}".format(self.grid_type))
        right, left = self.edges[1:], self.edges[:-1]
        self.centers = 0.5 * (left + right)
        self.widths = right - left
        self.is_linear = self.grid_type == 0

    def __repr__(self):
        return (f"grid_1D(mx={self.mx}, xb={self.xb}, xe={self.xe}, rim={self.rim}, "
                f"grid_type={self.grid_type}, centered={self.centered})")
