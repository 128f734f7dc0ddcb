"""CPU checks of the alt-ref filter's oracle (oracle/altref_ref.py, a
restatement of buildAltRef, ebiv/encoder.go:326-407) on cases whose answer
follows from the reference's rule alone."""
import numpy as np

import altref_ref


def _frame(w, h, y, cb, cr):
    cw, ch = (w + 1) // 2, (h + 1) // 2
    return (np.full(w * h, y, np.uint8).tobytes() + np.full(cw * ch, cb, np.uint8).tobytes()
            + np.full(cw * ch, cr, np.uint8).tobytes())


def test_short_window_gives_no_altref():
    f = _frame(32, 32, 100, 120, 130)
    assert altref_ref.build_altref([f, f], 32, 32, 8) is None
    assert altref_ref.build_altref([f, f, f, f], 32, 32, 2) is None


def test_identical_frames_average_to_the_head():
    f = _frame(37, 21, 77, 128, 5)
    assert altref_ref.build_altref([f] * 5, 37, 21, 8) == f


def test_disagreeing_frames_give_no_altref():
    a, b = _frame(48, 32, 10, 128, 128), _frame(48, 32, 200, 128, 128)
    assert altref_ref.build_altref([a, b, b, b], 48, 32, 8) is None


def test_rounded_average_within_the_sad_limit():
    # Luma 100 vs 105: SAD 5 per sample <= 6, accepted; (100 + 105 + 105 + 1) // 3 = 103.
    a, b = _frame(16, 16, 100, 10, 20), _frame(16, 16, 105, 13, 20)
    out = altref_ref.build_altref([a, b, b], 16, 16, 8)
    y = np.frombuffer(out, np.uint8)
    assert (y[:256] == 103).all() and (y[256:320] == (10 + 13 + 13 + 1) // 3).all() and (y[320:] == 20).all()
