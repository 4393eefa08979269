"""WCSPHSolver: weakly compressible SPH (eng/solver_sph_wc.py:6-132).

The reference's kernels read ``stiffness`` and ``viscosity`` from the solver object when
they are first compiled (eng/solver_sph_wc.py:12-15), so a scene script may change them
after construction.  Here they are properties: assigning one pushes both to the device
(``tsg_set_fluid``), and the next step uses the new value.
"""
import ctypes

from . import _native as nat
from .solver_sph_base import SPHBase


class WCSPHSolver(SPHBase):
    def __init__(self, particle_system):
        super().__init__(particle_system)
        m = self.ps.mat_fluid[0]
        self.density0 = m["density0"]
        self._viscosity = float(m["viscosity"])
        self._stiffness = float(m["stiffness"])
        self.exponent = m["exponent"]
        self.vsound = 60

    def calc_density(self):
        """Density summation, the reference's calc_density_task summed over every particle's
        neighbours (eng/solver_sph_wc.py:30-31): sum_j mass_j W(x_i - x_j), j != i, as a
        CUDA f64 tensor of particle_max_num values in the current particle order (the order
        of ``ps.field``).  The reference defines it but never calls it from a step; as there,
        the sum has no self term and dummy particles carry zero mass."""
        import torch
        out = torch.empty(self.ps.particle_max_num, dtype=torch.float64, device="cuda")
        self._call("tsg_density_sum", ctypes.c_void_p(out.data_ptr()))
        return out

    def _push(self):
        nat.check(self._lib.tsg_set_fluid(self._h, self._stiffness, self._viscosity), "tsg_set_fluid")

    @property
    def stiffness(self):
        return self._stiffness

    @stiffness.setter
    def stiffness(self, value):
        self._stiffness = float(value)
        self._push()

    @property
    def viscosity(self):
        return self._viscosity

    @viscosity.setter
    def viscosity(self, value):
        self._viscosity = float(value)
        self._push()
