"""CPU pins of the block-analysis oracle (oracle/transform_ref.py): its
forward DCT round-trips through the oracle's inverse within 3 (the
reference's TestDCTRoundTrip bound) and equals the formula restated in
test_oracle_known_answers; satd of a DC block is n*n times the value."""
import ctypes as C

import numpy as np

import ebiv_oracle
import transform_ref


def _inverse(coef, n):
    src = (C.c_int32 * (n * n))(*[int(v) for v in coef.ravel()])
    dst = (C.c_int32 * (n * n))()
    ebiv_oracle.lib().eo_inverse_dct(src, dst, n)
    return np.array(dst, dtype=np.int64).reshape(n, n)


def test_forward_dct_round_trip_and_formula():
    rng = np.random.default_rng(5)
    for n in (4, 8, 16):
        blocks = rng.integers(-255, 256, size=(50, n, n)).astype(np.int32)
        coef = transform_ref.forward_dct(blocks, n)
        c = transform_ref.dct_matrix(n)
        for b in range(50):
            want = (((c @ blocks[b].astype(np.int64) + 4096) >> 13) @ c.T + 4096) >> 13
            assert (coef[b] == want).all()
            assert np.abs(_inverse(coef[b], n) - blocks[b]).max() <= 3


def test_satd_of_flat_and_impulse_blocks():
    for n in (4, 8, 16):
        flat = np.full((1, n, n), 7, np.int32)
        assert transform_ref.satd(flat, n)[0] == 7 * n * n
        imp = np.zeros((1, n, n), np.int32)
        imp[0, 0, 0] = -3
        assert transform_ref.satd(imp, n)[0] == 3 * n * n
