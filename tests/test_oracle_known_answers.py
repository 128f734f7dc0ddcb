"""The CPU oracle pinned against the reference's own known-answer and
property tests (restated): sign-data-hiding level vectors
(ebiv/coded_test.go:483-548), rANS round trips (ebiv/rans_test.go:43-130),
transform / quantizer / zigzag properties (ebiv/transform_test.go:11-151).

The encoder side of each round trip is the product encoder; the decode side
is the oracle, so each test checks the two restatements against each other
and against the reference's stated invariants."""
import ctypes as C
import random

import numpy as np
import pytest

import ebiv_oracle
from govid_gb300 import _native

N_CTX = 72
ALPHABET = [3, 10, 10, 3, 2, 4, 8, 2, 16, 16, 16, 2] + [7] * 60


def _lib():
    return _native.lib()


def _encode_block(levels, n, plane=0, tx=0):
    lv = (C.c_int32 * (n * n))(*levels)
    stream = (C.c_uint8 * 65536)()
    ln = C.c_size_t()
    freqs = (C.c_uint32 * (N_CTX * 16))()
    used = (C.c_uint8 * N_CTX)()
    assert _lib().ebiv_encode_block(lv, n, plane, tx, stream, len(stream), C.byref(ln), freqs, used) == 0
    return list(lv), bytes(stream[: ln.value]), freqs, used


def _decode_block(stream, freqs, used, n, plane=0, tx=0):
    out = (C.c_int32 * (n * n))()
    L = ebiv_oracle.lib()
    st = L.eo_decode_block(stream, C.c_size_t(len(stream)), freqs, used, plane, tx, n, out)
    return st, list(out)


def _scan(n):
    order = (C.c_int * (n * n))()
    ebiv_oracle.lib().eo_zigzag(n, order)
    return list(order)


# TestSignDataHidingBlock's level patterns (ebiv/coded_test.go:484-492)
SDH_CASES = [
    [3, 0, 0, -2, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [-1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [1, 0, 0, 0, 0, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [2, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, -7],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [5, 4, 3, 2, 1, -1, -2, -3, -4, -5, 6, 7, 8, 9, 1, 1],
]


@pytest.mark.parametrize("case", range(len(SDH_CASES)))
def test_sign_data_hiding_known_answers(case):
    orig = SDH_CASES[case]
    n = 4
    scan = _scan(n)
    adj, stream, freqs, used = _encode_block(orig, n)

    def span(lv):
        nz = [i for i in range(n * n) if lv[scan[i]] != 0]
        return (nz[0], nz[-1]) if nz else (-1, -1)

    # adjustment never moves the first or last nonzero position
    assert span(adj) == span(orig)
    first, last = span(adj)
    if first >= 0 and last - first >= 4:
        parity = sum(abs(v) for v in adj) & 1
        assert parity == (1 if adj[scan[first]] < 0 else 0)
    st, got = _decode_block(stream, freqs, used, n)
    assert st == 0
    assert got == adj


def test_sign_data_hiding_random_blocks():
    rng = random.Random(17)
    for n in (4, 8, 16):
        for _ in range(60):
            lv = [0] * (n * n)
            for _ in range(rng.randint(0, n * n // 3)):
                lv[rng.randrange(n * n)] = rng.choice([-1, 1]) * rng.choice([1, 1, 1, 2, 3, 5, 9, 40, 300])
            adj, stream, freqs, used = _encode_block(lv, n, plane=0, tx={4: 0, 8: 1, 16: 2}[n])
            st, got = _decode_block(stream, freqs, used, n, plane=0, tx={4: 0, 8: 1, 16: 2}[n])
            assert st == 0 and got == adj


def _encode_tokens(toks):
    arr = (C.c_uint16 * (2 * len(toks)))(*[v for t in toks for v in t])
    stream = (C.c_uint8 * (len(toks) * 4 + 64))()
    ln = C.c_size_t()
    freqs = (C.c_uint32 * (N_CTX * 16))()
    used = (C.c_uint8 * N_CTX)()
    assert _lib().ebiv_encode_tokens(arr, len(toks), stream, len(stream), C.byref(ln), freqs, used) == 0
    return bytes(stream[: ln.value]), freqs, used


def test_rans_round_trip_random_streams():
    # TestRansRoundTrip: random token runs over every context round-trip.
    rng = random.Random(1)
    L = ebiv_oracle.lib()
    for _ in range(120):
        n = rng.randint(1, 4000)
        toks = []
        for _ in range(n):
            c = rng.randrange(N_CTX)
            toks.append((c, rng.randrange(ALPHABET[c])))
        stream, freqs, used = _encode_tokens(toks)
        ctxs = (C.c_int * n)(*[t[0] for t in toks])
        syms = (C.c_int * n)()
        assert L.eo_decode_symbols(stream, C.c_size_t(len(stream)), freqs, used, ctxs, n, syms) == 0
        assert list(syms) == [t[1] for t in toks]


def test_rans_single_symbol_context():
    toks = [(7, 0)] * 500  # TestRansSingleSymbolContext: ctxSign always 0
    stream, freqs, used = _encode_tokens(toks)
    n = len(toks)
    ctxs = (C.c_int * n)(*[7] * n)
    syms = (C.c_int * n)()
    assert ebiv_oracle.lib().eo_decode_symbols(stream, C.c_size_t(len(stream)), freqs, used, ctxs, n, syms) == 0
    assert set(syms) == {0}


def test_rans_underrun_and_unused_context_are_errors():
    stream, freqs, used = _encode_tokens([(3, 0), (3, 1), (3, 2)] * 10)
    L = ebiv_oracle.lib()
    n = 40
    ctxs = (C.c_int * n)(*[3] * n)
    syms = (C.c_int * n)()
    assert L.eo_decode_symbols(stream[:16], C.c_size_t(16), freqs, used, ctxs, n, syms) == 1
    ctxs2 = (C.c_int * 1)(5)
    assert L.eo_decode_symbols(stream, C.c_size_t(len(stream)), freqs, used, ctxs2, 1, syms) == 1


def test_normalized_tables_sum_to_total():
    # TestNormalizeFreqsSumsToTotal: every present symbol keeps a frequency.
    rng = random.Random(7)
    for _ in range(200):
        toks = []
        for c in (8, 9, 12, 30):
            for s in range(ALPHABET[c]):
                if rng.randrange(3) == 0:
                    toks += [(c, s)] * rng.randint(1, 3000)
        if not toks:
            continue
        _, freqs, used = _encode_tokens(toks)
        present = {}
        for c, s in toks:
            present.setdefault(c, set()).add(s)
        for c in range(N_CTX):
            f = list(freqs[c * 16: c * 16 + 16])
            if c in present:
                assert used[c] and sum(f) == 4096
                for s in range(ALPHABET[c]):
                    assert (f[s] > 0) == (s in present[c])


def _dct(n):
    m = (C.c_int32 * (n * n))()
    assert ebiv_oracle.lib().eo_dct_matrix(n, m) == 0
    return np.array(m, dtype=np.int64).reshape(n, n)


def test_dct_matrix_constants():
    # buildDCTMatrix (ebiv/transform.go:27-40) evaluated independently here.
    for n in (4, 8, 16):
        k = np.arange(n)[:, None]
        i = np.arange(n)[None, :]
        alpha = np.where(k == 0, np.sqrt(1.0 / n), np.sqrt(2.0 / n))
        c = alpha * np.cos((2 * i + 1) * k * np.pi / (2 * n)) * 8192
        want = np.sign(c) * np.floor(np.abs(c) + 0.5)
        frac = np.abs(np.abs(c) - np.floor(np.abs(c)) - 0.5)
        assert frac.min() > 1e-6  # no value sits on a rounding boundary
        assert (_dct(n) == want.astype(np.int64)).all()


def _inverse(coeffs, n):
    src = (C.c_int32 * (n * n))(*[int(v) for v in coeffs.ravel()])
    dst = (C.c_int32 * (n * n))()
    ebiv_oracle.lib().eo_inverse_dct(src, dst, n)
    return np.array(dst, dtype=np.int64).reshape(n, n)


def test_dct_round_trip_error_within_3():
    # TestDCTRoundTrip: forward (reference formula) then the oracle inverse.
    rng = np.random.default_rng(3)
    for n in (4, 8, 16):
        c = _dct(n)
        worst = 0
        for _ in range(300):
            src = rng.integers(-255, 256, size=(n, n)).astype(np.int64)
            acc = c @ src  # columns, int64 exact
            tmp = (acc + 4096) >> 13
            coef = (tmp @ c.T + 4096) >> 13
            back = _inverse(coef, n)
            worst = max(worst, int(np.abs(back - src).max()))
        assert worst <= 3


def test_inverse_dct_sparse_paths_match_full_transform():
    # The bounding-box and DC-only shortcuts equal the full separable product.
    rng = np.random.default_rng(11)
    for n in (4, 8, 16):
        c = _dct(n)
        for trial in range(200):
            coef = np.zeros((n, n), np.int64)
            r, q = rng.integers(1, n + 1), rng.integers(1, n + 1)
            if trial % 5 == 0:
                r = q = 1
            coef[:r, :q] = rng.integers(-3000, 3000, size=(r, q))
            tmp = ((c.T @ coef) + 4096) >> 13
            tmp = ((tmp + 2**31) % 2**32) - 2**31
            full = ((tmp @ c) + 4096) >> 13
            full = ((full + 2**31) % 2**32) - 2**31
            assert (_inverse(coef, n) == full).all()


def test_quant_steps_and_round_trip():
    # quantStep / newQuantizer (ebiv/quant.go:19-51) and TestQuantRoundTrip.
    L = ebiv_oracle.lib()
    for qp in range(64):
        dc, ac = C.c_int32(), C.c_int32()
        L.eo_quant_steps(qp, C.byref(dc), C.byref(ac))
        step = max(1, int(np.floor(2 ** (qp / 6) + 0.5)))
        assert ac.value == step
        assert dc.value == (max(1, int(np.floor(2 ** ((qp - 6) / 6) + 0.5))) if qp >= 6 else step)
        rng = np.random.default_rng(5 + qp)
        for c in rng.integers(-4000, 4001, size=200):
            for s in (ac.value, dc.value):
                lvl = (c * 8 + 3 * s) // (s * 8) if c >= 0 else -((-c * 8 + 3 * s) // (s * 8))
                assert abs(c - lvl * s) <= s


def test_zigzag_is_a_permutation_starting_at_dc():
    for n in (4, 8, 16):
        z = _scan(n)
        assert sorted(z) == list(range(n * n)) and z[0] == 0


def test_key_frames_from_chosen_levels_decode_in_the_oracle():
    # ebiv_encode_key_from_levels builds a key frame from given levels; the
    # oracle decodes it, and its wide-residual count sees the huge ones.
    from govid_gb300 import ebiv

    w, h = 48, 32
    mbs = 3 * 2
    small = np.zeros((mbs, 384), np.int32)
    small[:, 0] = 3
    small[:, 256] = -2
    ebiv_oracle.wide_residuals(True)
    st, planes = ebiv_oracle.decode_all([ebiv.encode_key_from_levels(w, h, 22, 0, small)])[0]
    assert st == 0 and ebiv_oracle.wide_residuals() == 0
    huge = small.copy()
    huge[::2, 0:16] = 32772
    st, planes = ebiv_oracle.decode_all([ebiv.encode_key_from_levels(w, h, 51, 0, huge)])[0]
    assert st == 0 and ebiv_oracle.wide_residuals() > 0
    with pytest.raises(ebiv.ErrArgument):
        ebiv.encode_key_from_levels(w, h, 22, 0, small[:-1])


# TestTileGridSplit's shapes (ebiv/tile_test.go:12-45): (mbCols, mbRows, cols, rows),
# grids larger than the frame included (newTileGrid clamps, ebiv/frame.go:87-102).
TILE_SPLITS = [(10, 8, 1, 1), (10, 8, 3, 2), (10, 8, 4, 4), (5, 5, 8, 8), (1, 1, 2, 2)]


def _with_tile_counts(pkt, cols, rows):
    """The packet with its coded header's one-byte tile-count varints replaced
    (codedHeader.appendTo, ebiv/frame.go:187-194)."""
    from govid_gb300 import ebiv

    b = ebiv.parse_frame_header(pkt)["body_offset"]
    assert pkt[b + 1] < 128 and pkt[b + 2] < 128 and cols < 128 and rows < 128
    return pkt[: b + 1] + bytes([cols, rows]) + pkt[b + 3:]


@pytest.mark.parametrize("split", TILE_SPLITS)
def test_tile_grid_split_decodes_and_clamps(split):
    # The encoder writes the clamped grid; the oracle decodes every grid to the
    # encoder's reconstruction. A header asking for more tiles than the
    # macroblock grid holds is corrupt: parsePayload reads cols*rows tile
    # records, then decodeCoded's grid check (ebiv/decode_intra.go:60-63) fails.
    from govid_gb300 import ebiv
    from helpers import encode_gen

    mbc, mbr, cols, rows = split
    cont, _, rec = encode_gen(16 * mbc, 16 * mbr, 3, ebiv.synth_pan, intra=20, gop=3, tiles=(cols, rows))
    pkts = [p.data for p in ebiv.Reader(cont).packets()]
    for p in pkts:
        b = ebiv.parse_frame_header(p)["body_offset"]
        assert (p[b + 1], p[b + 2]) == (min(cols, mbc), min(rows, mbr))
    got = ebiv_oracle.decode_all(pkts)
    assert [g[0] for g in got] == [0, 0, 0]
    assert [g[1] for g in got] == rec
    over = ebiv_oracle.decode_all([_with_tile_counts(p, min(cols, mbc) + 1, min(rows, mbr)) for p in pkts])
    assert over[0][0] == ebiv.ErrCorrupt.status
