"""Single-GPU annealing method (altar/altar/bayesian/CUDAAnnealing.py,
AnnealingMethod.py:55-147).

Each phase of a stage (cool, walk, resample) is a fixed sequence of C-ABI
launches whose stage-dependent inputs (β, scaling, Σ, the random-stream
epoch) live on the device.  After one eager stage has allocated every
buffer, the launches are captured into CUDA graphs and replayed for all
later stages: the whole stage as one graph when the sampler's walk is the
same every stage (plain Metropolis), else one graph per phase (the
delayed-acceptance walks change with per-stage host decisions).  The host
only reads β (and the stage report) once per stage.
"""
import ctypes
import logging
import time

import torch

from .. import _native
from ..device import stream_handle
from .coolingstep import CoolingStep

log = logging.getLogger("altar_gb300")


class CUDAAnnealing:
    def __init__(self, annealer, graphs=True, wid=0):
        self.annealer = annealer
        self.graphs = bool(graphs)
        self.wid = wid                              # worker id (the rank), as in the reference's workers
        self.step = None
        self.iteration = 0
        self.stream = None
        self._graphs = {}
        self._eager_done = set()
        self._last_bufs = None
        self.reports = []

    def initialize(self, application):
        self.stream = torch.cuda.Stream()
        return self

    @property
    def beta(self):
        return self.step.beta

    def start(self, annealer):
        self.iteration = 0
        if annealer.resume is not None:
            from ..simulations.checkpoint import Checkpoint
            model = annealer.model
            self.step = CoolingStep.alloc(samples=model.job.chains, parameters=model.parameters)
            arrays = Checkpoint.load(annealer.resume, model.job.chains, model.parameters)
            self.iteration = Checkpoint.restore(self.step, arrays)
            return self                            # the checkpoint carries the proposal scaling
        self.step = CoolingStep.start(annealer)
        annealer.sampler.prime(self.step)
        return self

    def top(self, annealer):
        annealer.model.top(step=self.step)
        return self

    def _eager(self):
        # a monitor that times the phases inside a stage (the Profiler) needs them launched one
        # by one: a replayed graph does not call back into the host
        return not self.graphs or getattr(self.annealer.dispatcher, "eager", False)

    def _phase(self, name, fn):
        """Run fn eagerly the first time (allocating its buffers), as a captured graph afterwards."""
        if self._eager() or name not in self._eager_done:
            self._eager_done.add(name)
            return fn()
        ex = self._graphs.get(name)
        if ex is None:
            s = stream_handle()
            _native.call("ag_graph_begin", s)
            try:
                fn()
            except Exception:
                dummy = ctypes.c_void_p()
                _native.load().ag_graph_end(s, ctypes.byref(dummy))
                raise
            handle = ctypes.c_void_p()
            _native.call("ag_graph_end", s, ctypes.byref(handle))
            ex = self._graphs[name] = handle
        _native.call("ag_graph_launch", ex, stream_handle())
        return None

    def fusable(self, annealer):
        """Whether the whole stage can replay as one graph."""
        return (not self._eager() and getattr(annealer.sampler, "static_walk", False)
                and ("cool" in self._eager_done or "stage" in self._graphs))

    def stage(self, annealer):
        """cool, walk and resample; one captured graph for the whole stage where possible."""
        if not self.fusable(annealer):
            self.cool(annealer)
            stats = self.walk(annealer)
            self.resample(annealer, stats)
            return self
        st = self.step.state
        if self._last_bufs is None:
            self._last_bufs = (st.scalars.clone(), st.counters.clone(), st.flags.clone())

        def run():
            annealer.scheduler.update(step=self.step)
            annealer.sampler.samplePosterior(annealer=annealer, step=self.step)
            for dst, src in zip(self._last_bufs, (st.scalars, st.counters, st.flags)):
                dst.copy_(src)
            annealer.sampler.resample(annealer=annealer, statistics=st.counters)

        self._eager_done.add("stage")           # the first fused stage is captured directly
        self._phase("stage", run)
        self._last = self._last_bufs
        self.iteration += 1
        return self

    def cool(self, annealer):
        self._phase("cool", lambda: annealer.scheduler.update(step=self.step))
        self.iteration += 1
        return self

    def walk(self, annealer):
        sampler = annealer.sampler
        sampler.prepare(annealer=annealer, step=self.step)
        run = lambda: sampler.samplePosterior(annealer=annealer, step=self.step)
        if sampler.capturable:
            self._phase("walk:" + sampler.mode_key(), run)
        else:
            run()
        return self.step.state.counters

    def resample(self, annealer, statistics):
        # report of the stage before the counters are cleared
        st = self.step.state
        self._last = (st.scalars.clone(), st.counters.clone(), st.flags.clone())
        self._phase("resample", lambda: annealer.sampler.resample(annealer=annealer, statistics=statistics))
        return self

    def bottom(self, annealer):
        scal, cnt, flags = (t.cpu() for t in self._last)
        acc, rej, unl = (int(v) for v in cnt)
        rep = {"stage": self.iteration, "time": time.perf_counter(), "beta": float(scal[0]),
               "dbeta": float(scal[1]),
               "cov": float(scal[2]), "scaling": float(self.step.state.scaling.item()),
               "accepted": acc, "rejected": rej, "unlikely": unl, "flags": int(flags[0])}
        rep.update(annealer.sampler.report())
        self.reports.append(rep)
        if rep["flags"] & _native.AG_DEV_ERR_TIMEOUT:
            raise RuntimeError("a device wait timed out during the stage")
        if rep["flags"] & _native.AG_DEV_ERR_NOT_SPD:
            log.warning("stage %d: scaled Σ not positive definite; diagonal proposal used", self.iteration)
        log.info("stage %(stage)d beta %(beta).6g cov %(cov).4g accepted %(accepted)d", rep)
        annealer.model.bottom(step=self.step)
        ck = annealer.checkpoint
        if ck is not None and ck.due(self.iteration):
            ck.save(ck.path, self.step, self.iteration)
        return self

    def forget_graphs(self):
        """Release the captured graphs; the next stage captures afresh (after a change of the
        sampler's settings that changes its launch sequence)."""
        for ex in self._graphs.values():
            _native.load().ag_graph_destroy(ex)
        self._graphs.clear()
        return self

    def finish(self, annealer):
        if annealer.archiver is not None:
            annealer.archiver.record(step=self.step)
        return self.forget_graphs()
