"""Philox4x32-10 (Salmon et al., SC 2011) and the draw conventions of the device kernels.

Oracle only (test infrastructure): reproduces, bit for bit, the uniforms the
GPU stage kernels draw, so that resampling counts and Metropolis decisions can
be compared exactly.
"""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)

STREAM_PRIOR, STREAM_PROPOSAL, STREAM_ACCEPT, STREAM_RESAMPLE = 0, 1, 2, 3


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 over uint32 counter arrays; returns four uint32 arrays."""
    c0, c1, c2, c3 = (np.asarray(c, dtype=np.uint64) & MASK32 for c in (c0, c1, c2, c3))
    c0, c1, c2, c3 = np.broadcast_arrays(c0, c1, c2, c3)
    k0 = np.uint64(int(k0) & 0xFFFFFFFF)
    k1 = np.uint64(int(k1) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & MASK32, lo1, (hi0 ^ c3 ^ k1) & MASK32, lo0
        k0 = (k0 + np.uint64(W0)) & MASK32
        k1 = (k1 + np.uint64(W1)) & MASK32
    return tuple(x.astype(np.uint32) for x in (c0, c1, c2, c3))


def draw(seed, unit, sub, stream, step, epoch):
    seed = int(seed)
    c2 = (np.uint64(stream) << np.uint64(24)) | (np.asarray(step, dtype=np.uint64) & np.uint64(0xFFFFFF))
    return philox4x32_10(unit, sub, c2, epoch, seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)


def bits53(a, b):
    return ((a.astype(np.uint64) >> np.uint64(5)) << np.uint64(26)) | (b.astype(np.uint64) >> np.uint64(6))


def u01_closed_open(a, b):
    return bits53(a, b).astype(np.float64) * 2.0 ** -53


def u01_open_closed(a, b):
    return (bits53(a, b) + np.uint64(1)).astype(np.float64) * 2.0 ** -53


def normal_pair(r):
    u1 = u01_open_closed(r[0], r[1])
    u2 = u01_closed_open(r[2], r[3])
    rad = np.sqrt(-2.0 * np.log(u1))
    return rad * np.cos(2.0 * np.pi * u2), rad * np.sin(2.0 * np.pi * u2)


def proposal_normals(seed, n, p, step, epoch):
    """N(0,1) draws of the proposal kernel: (n, p)."""
    z = np.empty((n, p))
    units = np.arange(n, dtype=np.uint64)
    for j in range(0, p, 2):
        z0, z1 = normal_pair(draw(seed, units, j >> 1, STREAM_PROPOSAL, step, epoch))
        z[:, j] = z0
        if j + 1 < p:
            z[:, j + 1] = z1
    return z


def accept_uniforms(seed, n, step, epoch):
    r = draw(seed, np.arange(n, dtype=np.uint64), 0, STREAM_ACCEPT, step, epoch)
    return u01_open_closed(r[0], r[1])


def resample_uniforms(seed, n, epoch):
    r = draw(seed, np.arange(n, dtype=np.uint64), 0, STREAM_RESAMPLE, 0, epoch)
    return u01_closed_open(r[0], r[1])


def prior_uniforms(seed, n, p, attempt):
    u = np.empty((n, p))
    units = np.arange(n, dtype=np.uint64)
    for j in range(p):
        r = draw(seed, units, j, STREAM_PRIOR, 0, attempt)
        u[:, j] = u01_closed_open(r[0], r[1])
    return u
