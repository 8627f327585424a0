"""The allocation-free COV schedule agrees with the workspace version.

ag_cov_schedule_noalloc serves callers that cannot allocate device memory when
they run a stage (for example under a fixed device-memory budget): it keeps its
scratch in an array inside the library instead of a caller workspace.  This file is collected last so that a failure
here leaves every other test already run; it passes alone and after the rest.
Tolerance: the β schedule tests' 1e-12 relative on β, δβ, COV and the weights
(the two entry points run the same kernels, so the results are expected to be
identical).
"""
import numpy as np
import pytest
import torch

from altar_gb300 import _native
from altar_gb300.bayesian.coolingstep import StageState
from altar_gb300.device import ptr, stream_handle, workspace

pytestmark = pytest.mark.gpu


def _run(entry, llk, beta0, n):
    st = StageState(n, 2)
    st.beta.fill_(beta0)
    d = torch.from_numpy(llk).cuda()
    if entry == "ag_cov_schedule":
        ws = workspace(_native.load().ag_cov_workspace_bytes(n))
        _native.call(entry, st.struct, ptr(d), n, 1.0, 0.01, ptr(ws), ws.numel(), stream_handle())
    else:
        _native.call(entry, st.struct, ptr(d), n, 1.0, 0.01, stream_handle())
    torch.cuda.synchronize()
    return st.scalars.cpu().numpy()[:3].copy(), st.w.cpu().numpy().copy()


def test_noalloc_schedule_matches_workspace_version(cuda):
    rng = np.random.default_rng(11)
    cases = [(rng.normal(-3e4, 1e3, 40000), 0.0), (-np.exp(rng.uniform(0, 12, 9000)), 0.2)]
    for llk, beta0 in cases:                       # two calls in a row share the library's scratch
        n = llk.size
        ref_s, ref_w = _run("ag_cov_schedule", llk, beta0, n)
        got_s, got_w = _run("ag_cov_schedule_noalloc", llk, beta0, n)
        np.testing.assert_allclose(got_s, ref_s, rtol=1e-12, atol=0)
        np.testing.assert_allclose(got_w, ref_w, rtol=1e-12, atol=1e-300)


def test_noalloc_at_the_chain_limit(cuda):
    """At ag_cov_schedule_noalloc_max_chains() chains the per-block partials fill the whole
    fixed scratch array (an undersized array would show here first)."""
    n = _native.load().ag_cov_schedule_noalloc_max_chains()
    llk = np.random.default_rng(5).normal(-2e4, 3e2, n)
    for beta0 in (0.0, 0.3):                       # two calls in a row at the limit
        ref_s, ref_w = _run("ag_cov_schedule", llk, beta0, n)
        got_s, got_w = _run("ag_cov_schedule_noalloc", llk, beta0, n)
        np.testing.assert_allclose(got_s, ref_s, rtol=1e-12, atol=0)
        np.testing.assert_allclose(got_w, ref_w, rtol=1e-12, atol=1e-300)


def test_noalloc_rejects_too_many_chains(cuda):
    lib = _native.load()
    big = lib.ag_cov_schedule_noalloc_max_chains() + 1
    st = StageState(4, 2)
    rc = lib.ag_cov_schedule_noalloc(st.struct, ptr(st.w), big, 1.0, 0.01, stream_handle())
    assert rc == 4 and "chains" in _native.last_error()
