"""Run log of the sketch-and-precondition solvers.

Same fields and amortisation rule as ``SketchAndPrecondLog`` in
``parla/comps/determiter/logging.py:4-94``, so code that reads the
reference's logs reads these unchanged.  Phase times are wall-clock seconds
taken with the device synchronised at each phase boundary.
"""
import numpy as np


class SketchAndPrecondLog:

    def __init__(self):
        self.time_sketch = 0.0
        self.time_factor = 0.0
        self.time_presolve = 0.0
        self.time_convert = 0.0
        self._time_setup = 0.0
        self.time_iterate = 0.0
        self.times = None
        self.errors = None
        self.error_desc = """Fill in."""
        # additions: LSQR stop code and iteration count of the device solve
        self.istop = None
        self.itn = None

    @property
    def time_setup(self):
        self._time_setup = self.time_sketch + self.time_factor + self.time_convert
        return self._time_setup

    def wrap_up(self, iter_errors, init_error):
        """errors = [init, per-iteration...]; iterating time spread evenly (``:72-93``)."""
        iters = iter_errors.size
        setup = self.time_setup
        ramp = np.linspace(0, self.time_iterate, iters, endpoint=True)
        self.times = np.concatenate(([setup], setup + self.time_presolve + ramp))
        self.errors = np.concatenate(([init_error], iter_errors))
