"""Final-state archiver (altar/altar/simulations/Recorder.py:17-58).

Writes the final sample θ, the parameter covariance Σ and the posterior
log-likelihoods as text files, one row per chain, and at initialisation the
sample layout (``parameters.csv``: name, count, offset of each parameter set),
which the reference's models write themselves (models/cdm/cdm/CDM.py:358-380).
"""
import numpy as np


class Recorder:
    def __init__(self, theta="theta.txt", sigma="sigma.txt", llk="llk.txt", parameters="parameters.csv"):
        self.theta, self.sigma, self.llk, self.parameters = theta, sigma, llk, parameters

    def initialize(self, application):
        if self.parameters:
            application.model.meta(self.parameters)
        return self

    def record(self, step, **kwds):
        np.savetxt(self.theta, step.theta.cpu().numpy())
        np.savetxt(self.sigma, step.sigma.cpu().numpy())
        np.savetxt(self.llk, step.posterior.cpu().numpy())
        return self
