"""Chain sharding across ranks (altar/altar/bayesian/MPIAnnealing.py:106-269).

The reference's MPI annealing scatters the chains of one population across
workers and gathers them at the manager every stage.  Here every rank keeps the
whole population (θ, prior, data and posterior log-likelihoods: N (p + 3)
doubles, 3.4 MB at 32,768 chains of 10 parameters), walks only its own block of
rows, and the blocks are exchanged once per stage:

  * after the walk, an all-gather of every rank's rows (``ChainShards.gather``)
    and an all-reduce of the accept/reject counters (``ChainShards.sum``), so
    that the scaling adaptation sees the whole population's acceptance;
  * the cool phase (COV β, weighted Σ, multinomial resampling) then runs on the
    whole population on every rank, from identical inputs with fixed-order
    kernels, so every rank holds the same β, Σ and resampled population.

The proposal and accept streams are keyed by the global chain index (the stage
state's ``chain0``), so a sharded run draws exactly what one process draws and
reproduces it bit for bit.  (The reference instead seeds each worker's
generator separately, MPIAnnealing.py:39-41.)  The collectives work on any
torch.distributed backend: NCCL for device tensors, gloo for host tensors.
"""
import torch

from .annealing import CUDAAnnealing


class ChainShards:
    """Contiguous equal blocks of a population's rows, one per rank."""

    def __init__(self, dist=None, group=None):
        if dist is None:
            import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def bounds(self, n):
        """(first row, rows) of this rank's block of an n-chain population."""
        if n % self.world:
            raise ValueError(f"{n} chains do not split evenly over {self.world} ranks")
        m = n // self.world
        return self.rank * m, m

    def gather(self, full, *more):
        """Every rank's block of each row-major tensor (rows first), in place: after the call
        every rank holds the blocks of all ranks.  The tensors are packed into one buffer so
        that a stage needs one collective."""
        tensors = (full,) + more
        n = full.shape[0]
        c0, m = self.bounds(n)
        widths = [t[0].numel() if t.dim() > 1 else 1 for t in tensors]
        w = sum(widths)
        local = torch.empty(m, w, dtype=full.dtype, device=full.device)
        col = 0
        for t, k in zip(tensors, widths):
            local[:, col:col + k] = t[c0:c0 + m].reshape(m, k)
            col += k
        out = torch.empty(self.world * m, w, dtype=full.dtype, device=full.device)
        self.dist.all_gather_into_tensor(out, local, group=self.group)
        col = 0
        for t, k in zip(tensors, widths):
            t.copy_(out[:, col:col + k].reshape(t.shape))
            col += k
        return tensors

    def sum(self, t):
        """All-reduce (sum) in place."""
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        return t


class _Block:
    """A rank's rows of the population as a CoolingStep for the sampler: views of the whole
    population's tensors and a stage-state struct with the block's global first chain."""

    def __init__(self, step, c0, m):
        self.theta = step.theta[c0:c0 + m]
        self.prior = step.prior[c0:c0 + m]
        self.data = step.data[c0:c0 + m]
        self.posterior = step.posterior[c0:c0 + m]
        self.state = step.state.view(chain0=c0)

    @property
    def samples(self):
        return self.theta.shape[0]

    @property
    def parameters(self):
        return self.theta.shape[1]

    @property
    def beta(self):
        return float(self.state.beta.item())


class ShardedAnnealing(CUDAAnnealing):
    """CUDAAnnealing over a population split across ranks: each rank walks its block of
    chains; the cool and resample phases run on the whole (gathered) population."""

    def __init__(self, annealer, shards, graphs=True):
        super().__init__(annealer, graphs=graphs, wid=shards.rank)
        self.shards = shards
        self.block = None

    def fusable(self, annealer):
        return False                            # the walk is followed by collectives

    def start(self, annealer):
        super().start(annealer)
        c0, m = self.shards.bounds(self.step.samples)
        self.block = _Block(self.step, c0, m)
        return self

    def walk(self, annealer):
        sampler = annealer.sampler
        if not getattr(sampler, "shardable", False):
            raise NotImplementedError(f"{type(sampler).__name__} cannot walk a sharded population")
        block = self.block
        sampler.prepare(annealer=annealer, step=block)
        run = lambda: sampler.samplePosterior(annealer=annealer, step=block)
        if sampler.capturable:
            self._phase("walk:" + sampler.mode_key(), run)
        else:
            run()
        step = self.step
        self.shards.gather(step.theta, step.prior, step.data, step.posterior)
        self.shards.sum(step.state.counters)
        return step.state.counters
