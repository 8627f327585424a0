"""δβ solver by iterative grid search (altar/altar/bayesian/Grid.py:19-63,
altar/lib/libaltar/bayesian/COV.cc:222-368), evaluated on the GPU.

The median of the data log-likelihood, the 11-point grid refinement and the
final importance weights all run on the device (ag_cov_schedule); β and COV
stay in the stage state.
"""
from .. import _native
from ..device import ptr, stream_handle, workspace


class Grid:
    def __init__(self, tolerance=0.01, maxiter=10 ** 3):
        self.tolerance = float(tolerance)
        self.maxiter = int(maxiter)
        self.target = 1.0
        self._ws = None
        self._ws_bytes = 0

    def initialize(self, application, scheduler):
        self.target = scheduler.target
        return self

    def solve(self, llk, weight, step):
        """Advance step.state.beta and fill the normalised weights (device)."""
        n = llk.shape[0]
        need = _native.load().ag_cov_workspace_bytes(n)
        if need > self._ws_bytes:
            self._ws, self._ws_bytes = workspace(need), need
        _native.call("ag_cov_schedule", step.state.struct, ptr(llk), n, self.target, self.tolerance,
                     ptr(self._ws), self._ws_bytes, stream_handle())
        return step.state.beta, step.state.dbeta_cov
