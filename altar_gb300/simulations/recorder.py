"""Final-state archiver (altar/altar/simulations/Recorder.py:17-58).

Writes the final sample θ, the parameter covariance Σ and the posterior
log-likelihoods as text files, one row per chain.
"""
import numpy as np


class Recorder:
    def __init__(self, theta="theta.txt", sigma="sigma.txt", llk="llk.txt"):
        self.theta, self.sigma, self.llk = theta, sigma, llk

    def initialize(self, application):
        return self

    def record(self, step, **kwds):
        np.savetxt(self.theta, step.theta.cpu().numpy())
        np.savetxt(self.sigma, step.sigma.cpu().numpy())
        np.savetxt(self.llk, step.posterior.cpu().numpy())
        return self
