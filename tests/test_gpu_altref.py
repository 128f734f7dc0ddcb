"""The GPU alt-ref temporal filter (ebivgpu_altref_build) against its oracle
(oracle/altref_ref.py, buildAltRef, ebiv/encoder.go:326-407), bit-exact, on
the reference test's hold-under-noise clip, odd sizes, and moving sprites
where only some blocks agree with the GOP head."""
import pytest

import altref_ref
from govid_gb300 import ebiv

from helpers import noisy_gen

pytestmark = pytest.mark.gpu


def _check(a, frames, w, h, window):
    want = altref_ref.build_altref(frames, w, h, window)
    got = a.build(frames, w, h, window)
    assert (got is None) == (want is None)
    assert got == want


@pytest.mark.parametrize("w,h", [(128, 96), (37, 21), (65, 49)])
def test_hold_under_noise(gpu_required, w, h):
    # TestAltRefGoldenOverride's generator (ebiv/coded_test.go:664-674)
    frames = [noisy_gen(w, h, i) for i in range(10)]
    a = ebiv.AltRef()
    for window in (3, 8, 10):
        _check(a, frames, w, h, window)
    assert a.build(frames, w, h, 8) is not None


def test_moving_sprites_partial_agreement(gpu_required):
    sc = ebiv.Scene(ebiv.SceneSpec(width=1280, height=720, seed=5, sprites=12, noise_y16=16, noise_c16=8))
    frames = [sc.render(i) for i in range(8)]
    a = ebiv.AltRef()
    _check(a, frames, 1280, 720, 8)
    assert 0 < a.accepted < 7 * 80 * 45  # some blocks agree, the moving ones do not
    # two calls in a row on one handle, then a smaller window
    _check(a, frames, 1280, 720, 8)
    _check(a, frames, 1280, 720, 4)


def test_no_altref_cases(gpu_required):
    a = ebiv.AltRef()
    f0, f1 = ebiv.synth_frame(64, 48, 1), ebiv.synth_frame(64, 48, 2)
    assert a.build([f0, f0], 64, 48, 8) is None  # window below 3
    _check(a, [f0, f1, f1, f1], 64, 48, 8)
