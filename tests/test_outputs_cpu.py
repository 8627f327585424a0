"""Output formats written by the host side (no GPU): the sample layout file."""
import csv

from altar_gb300.distributions import Uniform
from altar_gb300.models import Bayesian, Contiguous


def test_parameters_csv_layout(tmp_path):
    """parameters.csv holds name, count, offset per parameter set, as the reference's
    models write it (models/cdm/cdm/CDM.py:358-380)."""
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 1e4))),
             "opening": Contiguous(1, Uniform((-50, 50))), "a": Contiguous(3, Uniform((100, 3000))),
             "omega": Contiguous(3, Uniform((-90, 90)))}
    model = Bayesian(psets=psets)
    offset = 0
    for pset in psets.values():
        offset += pset.initialize(model=model, offset=offset)
    path = tmp_path / "parameters.csv"
    model.meta(str(path))
    with open(path, newline="") as f:
        rows = list(csv.reader(f))
    assert rows == [["name", "count", "offset"], ["location", "2", "0"], ["depth", "1", "2"],
                    ["opening", "1", "3"], ["a", "3", "4"], ["omega", "3", "7"]]
