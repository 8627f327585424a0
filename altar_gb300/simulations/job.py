"""Job parameters (altar/altar/simulations/Job.py:18-46).

Same names and defaults as the reference; ``gpus`` is the number of GPUs per
task and this implementation runs one task on one GPU.
"""
from dataclasses import dataclass


@dataclass
class Job:
    name: str = "sample"
    hosts: int = 1
    tasks: int = 1
    gpus: int = 1
    chains: int = 1
    steps: int = 20
    tolerance: float = 1.0e-3

    def initialize(self, application):
        """Validate the machine layout (Job.py:62-134): one task on one GPU."""
        if self.hosts != 1 or self.tasks != 1:
            raise ValueError("this implementation runs one task on one host")
        if self.gpus < 1:
            raise ValueError("the GB300 path needs gpus >= 1; there is no CPU strategy")
        if self.chains < 2:
            raise ValueError("CATMIP needs at least two chains")
        return self
