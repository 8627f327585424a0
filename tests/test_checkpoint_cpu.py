"""Checkpoint files: round trip of the stage arrays and the shape check (host only)."""
import types

import numpy as np
import pytest
import torch

from altar_gb300.simulations.checkpoint import Checkpoint


def _step(n=6, p=3):
    g = torch.Generator().manual_seed(0)
    st = types.SimpleNamespace(scalars=torch.rand(8, generator=g, dtype=torch.float64),
                               sigma=torch.rand(p, p, generator=g, dtype=torch.float64),
                               epoch=torch.tensor([7], dtype=torch.int32))
    return types.SimpleNamespace(theta=torch.rand(n, p, generator=g, dtype=torch.float64),
                                 prior=torch.rand(n, generator=g, dtype=torch.float64),
                                 data=torch.rand(n, generator=g, dtype=torch.float64),
                                 posterior=torch.rand(n, generator=g, dtype=torch.float64), state=st)


def test_round_trip(tmp_path):
    step = _step()
    path = str(tmp_path / "ck.npz")
    Checkpoint.save(path, step, 12)
    z = Checkpoint.load(path, 6, 3)
    assert int(z["iteration"]) == 12 and int(z["epoch"][0]) == 7
    np.testing.assert_array_equal(z["theta"], step.theta.numpy())
    np.testing.assert_array_equal(z["scalars"], step.state.scalars.numpy())
    assert Checkpoint(path, every=3).due(9) and not Checkpoint(path, every=3).due(10)


def test_shape_mismatch_rejected(tmp_path):
    path = str(tmp_path / "ck.npz")
    Checkpoint.save(path, _step(), 1)
    with pytest.raises(ValueError, match="samples x parameters"):
        Checkpoint.load(path, 5, 3)
