"""Annealing controller (altar/altar/bayesian/Annealer.py:21-187).

posterior(model): start from the prior at β = 0, then while β + tolerance < 1:
top → cool (β, Σ, resample) → walk (Metropolis) → resample (scaling) → bottom.
"""
import torch

from .annealing import CUDAAnnealing
from .cov import COV
from .metropolis import Metropolis
from .notifier import Notifier


class Annealer:
    def __init__(self, sampler=None, scheduler=None, dispatcher=None, archiver=None, graphs=True,
                 checkpoint=None, resume=None, shards=None):
        """checkpoint: a simulations.Checkpoint written after every ``every`` stages;
        resume: path of a checkpoint to continue from instead of sampling the prior;
        shards: a bayesian.ChainShards to split the population's walk across ranks."""
        self.sampler = sampler if sampler is not None else Metropolis()
        self.scheduler = scheduler if scheduler is not None else COV()
        self.dispatcher = dispatcher if dispatcher is not None else Notifier()
        self.archiver = archiver
        self.graphs = graphs
        self.checkpoint = checkpoint
        self.resume = resume
        self.shards = shards
        self.worker = None
        self.model = None

    def initialize(self, application):
        self.dispatcher.initialize(application=application)
        self.sampler.initialize(application=application)
        self.scheduler.initialize(application=application)
        if self.archiver is not None:
            self.archiver.initialize(application=application)
        if self.shards is not None:
            from .sharding import ShardedAnnealing
            self.worker = ShardedAnnealing(self, self.shards, graphs=self.graphs).initialize(application)
        else:
            wid = torch.distributed.get_rank() if torch.distributed.is_initialized() else 0
            self.worker = CUDAAnnealing(annealer=self, graphs=self.graphs, wid=wid).initialize(application)
        for monitor in getattr(application, "monitors", {}).values():
            monitor.initialize(application=application)
            self.dispatcher.register(monitor=monitor)
        return self

    def posterior(self, model, max_stages=10 ** 6):
        self.model = model
        tolerance = model.job.tolerance
        worker, d = self.worker, self.dispatcher
        with torch.cuda.stream(worker.stream):
            d.notify(event=d.start, controller=self)
            worker.start(annealer=self)
            stages = 0
            while worker.beta + tolerance < 1 and stages < max_stages:
                d.notify(event=d.betaStart, controller=self)
                worker.top(annealer=self)
                if worker.fusable(self):
                    # the whole stage replays as one graph; the phase events mark its launch
                    worker.stage(annealer=self)
                    for ev in (d.walkChainsStart, d.walkChainsFinish, d.resampleStart, d.resampleFinish):
                        d.notify(event=ev, controller=self)
                else:
                    worker.cool(annealer=self)
                    d.notify(event=d.walkChainsStart, controller=self)
                    statistics = worker.walk(annealer=self)
                    d.notify(event=d.walkChainsFinish, controller=self)
                    d.notify(event=d.resampleStart, controller=self)
                    worker.resample(annealer=self, statistics=statistics)
                    d.notify(event=d.resampleFinish, controller=self)
                worker.bottom(annealer=self)
                d.notify(event=d.betaFinish, controller=self)
                stages += 1
            worker.finish(annealer=self)
            d.notify(event=d.finish, controller=self)
            torch.cuda.current_stream().synchronize()
        self.model = None
        return 0
