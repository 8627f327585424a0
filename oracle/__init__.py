"""CPU oracle for the CATMIP hot path (test infrastructure only).

This package restates, in numpy FP64 (and in plain C under ``oracle/csrc``),
the reference algorithms that the CUDA library replaces.  It exists to check
the product and to time a CPU baseline; the product path never imports it.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its
``cpu_baseline`` leg and ``--impl reference`` arm) may use it.

Pinning:
  * CDM forward model: pinned against the Matlab golden vectors of the
    reference test ``models/cdm/tests/libcdm.py:27-46`` and against outputs
    of the reference ``models/cdm/cdm/libcdm.py`` itself (fixtures in
    ``tests/golden`` and the script that generated them).
  * Mogi, Gaussian log-likelihood, Uniform prior, Metropolis, COV grid
    solver, weighted covariance and multinomial resampling: restated from
    the cited reference lines; the reference needs pyre and GSL, which are
    not available, so these are pinned only by closed-form known answers
    (parity unpinned against GSL's RNG streams, histogram binning order and
    heap-sort tie order).
"""
