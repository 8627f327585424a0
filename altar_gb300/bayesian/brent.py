"""δβ solver by Brent's minimiser (altar/altar/bayesian/Brent.py:19-63,
altar/lib/libaltar/bayesian/COV.cc:58-219), evaluated on the GPU.

Same set-up as the reference: minimise (COV(δβ) − target)² over
[0, 1 − β] starting from the guess δβ = 5e-5, skip straight to β = 1 when the
full step already meets the target, stop when the COV of the latest point is
within ``tolerance`` of the target or after ``maxiter`` iterations, and keep
the best point.  The reference iterates GSL's Brent minimiser; the device
kernel restates Brent's published method (1973, procedure localmin).  At most
128 iterations run on the device per stage (a larger ``maxiter`` is capped
there); the median, every COV evaluation and the final weights are device
kernels, and β and COV stay in the stage state (ag_cov_schedule_brent).
"""
from .. import _native
from ..device import ptr, stream_handle, workspace


class Brent:
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
        _native.call("ag_cov_schedule_brent", step.state.struct, ptr(llk), n, self.target, self.tolerance,
                     self.maxiter, ptr(self._ws), self._ws_bytes, stream_handle())
        return step.state.beta, step.state.dbeta_cov
