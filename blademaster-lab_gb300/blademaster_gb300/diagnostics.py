"""Kinetic, elastic and gravitational energy of the material state.

diagnostics.Metrics (diagnostics.py:6-48): the same columns and ``read()``,
computed by bm_metrics on the device.  The three energies are exact sums of
the per-particle float32 terms (one rounding at the end), so repeated reads
of one state agree to the bit, which the reference's float atomics do not
promise.
"""

import numpy as np

from . import _native


class Metrics:
    columns = ["kinetic_J", "gravity_J", "elastic_diagnostic_J", "max_speed_m_s", "max_z_m", "min_det_F"]

    def __init__(self, solver):
        import torch

        self.s = solver
        self.array = torch.zeros(6, dtype=torch.float64, device=solver.device)

    def read(self):
        """float32 array of the six columns for the solver's current state."""
        s = self.s
        _native.check(s._lib.bm_metrics(s._handle, self.array.data_ptr(), s._stream))
        return self.array.cpu().numpy().astype(np.float32)
