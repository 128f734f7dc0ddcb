"""TEST INFRASTRUCTURE — the encoder's block analysis restated in numpy.

forwardDCT and satd (ebiv/transform.go:44-119): the separable 2^13-scaled
DCT-II with int64 accumulation, a rounding shift by 13 and Go's int32
narrowing after each pass; and the sum of absolute values of the 2-D
Walsh-Hadamard transform (int32 butterflies, wrapping like Go's int32).
The DCT matrices come from the C++ oracle (eo_dct_matrix, buildDCTMatrix,
ebiv/transform.go:27-40), which tests/test_oracle_known_answers.py checks
against the formula.  The checker for ebivgpu_fdct_satd; nothing in the
product imports it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

import ebiv_oracle


def dct_matrix(n: int) -> np.ndarray:
    m = (C.c_int32 * (n * n))()
    assert ebiv_oracle.lib().eo_dct_matrix(n, m) == 0
    return np.array(m, dtype=np.int64).reshape(n, n)


def _i32(a: np.ndarray) -> np.ndarray:
    return ((a + (1 << 31)) % (1 << 32) - (1 << 31)).astype(np.int64)


def forward_dct(blocks: np.ndarray, n: int) -> np.ndarray:
    """blocks: (count, n, n) int32 residuals -> (count, n, n) int32 coefficients."""
    c = dct_matrix(n)
    src = blocks.astype(np.int64)
    tmp = _i32((np.einsum("ki,bij->bkj", c, src) + 4096) >> 13)
    out = _i32((np.einsum("bkj,mj->bkm", tmp, c) + 4096) >> 13)
    return out.astype(np.int32)


def _fwht_lines(t: np.ndarray, n: int) -> np.ndarray:
    """fwht (ebiv/transform.go:108-119) along the last axis, int32 wrap."""
    t = t.copy()
    span = 1
    while span < n:
        for i in range(0, n, span << 1):
            x = t[..., i:i + span].copy()
            y = t[..., i + span:i + 2 * span].copy()
            t[..., i:i + span] = _i32(x + y)
            t[..., i + span:i + 2 * span] = _i32(x - y)
        span <<= 1
    return t


def satd(blocks: np.ndarray, n: int) -> np.ndarray:
    """blocks: (count, n, n) int32 -> (count,) int64 sums of |Hadamard|."""
    t = _fwht_lines(blocks.astype(np.int64), n)               # rows
    t = _fwht_lines(t.transpose(0, 2, 1), n).transpose(0, 2, 1)  # columns
    return np.abs(t).sum(axis=(1, 2)).astype(np.int64)
