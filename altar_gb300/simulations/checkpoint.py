"""Per-stage checkpoint and restart of the annealing state.

No counterpart in the reference: its annealing method starts every run from the
prior (altar/altar/bayesian/AnnealingMethod.py:65-70).  A checkpoint holds what
the next stage reads: θ, the prior/data/posterior log-likelihoods, β, δβ, COV,
the proposal scaling, Σ, the random-stream epoch and the stage count.  Every
random draw is keyed by (seed, epoch, step), so a run resumed from the
checkpoint of stage k repeats, with the same seed, the stages an uninterrupted
run makes after stage k.  Sampler state beyond the scaling (the learned
surrogate of the delayed-acceptance sampler) is not saved; such a sampler
refits after a restart.
"""
import os

import numpy as np
import torch

from ..device import DEVICE

FORMAT = 1


class Checkpoint:
    def __init__(self, path, every=1):
        self.path = path
        self.every = max(1, int(every))

    def initialize(self, application):
        return self

    def due(self, iteration):
        return iteration % self.every == 0

    @staticmethod
    def save(path, step, iteration):
        st = step.state
        arrays = dict(format=np.int64(FORMAT), iteration=np.int64(iteration),
                      theta=step.theta.cpu().numpy(), prior=step.prior.cpu().numpy(),
                      data=step.data.cpu().numpy(), posterior=step.posterior.cpu().numpy(),
                      scalars=st.scalars.cpu().numpy(), sigma=st.sigma.cpu().numpy(),
                      epoch=st.epoch.cpu().numpy())
        tmp = path + ".tmp.npz"
        np.savez(tmp, **arrays)
        os.replace(tmp, path)                      # a reader never sees a half-written file
        return path

    @staticmethod
    def load(path, samples, parameters):
        """Arrays of a checkpoint, checked against the run's shape."""
        with np.load(path) as z:
            if int(z["format"]) != FORMAT:
                raise ValueError(f"{path}: checkpoint format {int(z['format'])}, expected {FORMAT}")
            out = {k: z[k] for k in z.files}
        if out["theta"].shape != (samples, parameters):
            raise ValueError(f"{path}: checkpoint holds {out['theta'].shape} samples x parameters, "
                             f"the run has ({samples}, {parameters})")
        return out

    @staticmethod
    def restore(step, arrays):
        """Overwrite a freshly allocated CoolingStep with a checkpoint's arrays."""
        dev = dict(device=DEVICE)
        step.theta.copy_(torch.from_numpy(arrays["theta"]).to(**dev))
        step.prior.copy_(torch.from_numpy(arrays["prior"]).to(**dev))
        step.data.copy_(torch.from_numpy(arrays["data"]).to(**dev))
        step.posterior.copy_(torch.from_numpy(arrays["posterior"]).to(**dev))
        st = step.state
        st.scalars.copy_(torch.from_numpy(arrays["scalars"]).to(**dev))
        st.sigma.copy_(torch.from_numpy(arrays["sigma"]).to(**dev))
        st.epoch.copy_(torch.from_numpy(arrays["epoch"]).to(**dev))
        return int(arrays["iteration"])
