"""TEST INFRASTRUCTURE — the encoder's alt-ref temporal filter restated in numpy.

buildAltRef (ebiv/encoder.go:326-407): the golden-override image of a GOP is
the GOP head averaged, per 16x16 luma block, with every window frame whose
block agrees with the head's (luma SAD at most altRefBlockSAD = 6 per
sample, ebiv/encoder.go:320-322); the chroma co-located with a block
([bx/2, min(CW, (bx+bw+1)/2)) x [by/2, ...)) follows the block's decision.
Each sample is (sum + count/2) // count.  Returns None when the window is
below 3 frames or no block of any frame was accepted.

The checker for the GPU filter (ebivgpu_altref_build); nothing in the
product imports it.
"""
from __future__ import annotations

import numpy as np


def planes(packed: bytes, w: int, h: int):
    cw, ch = (w + 1) // 2, (h + 1) // 2
    a = np.frombuffer(packed, np.uint8)
    return (a[: w * h].reshape(h, w), a[w * h: w * h + cw * ch].reshape(ch, cw),
            a[w * h + cw * ch: w * h + 2 * cw * ch].reshape(ch, cw))


def build_altref(frames: list[bytes], w: int, h: int, window: int):
    n = min(window, len(frames))
    if n < 3:
        return None
    cw, ch = (w + 1) // 2, (h + 1) // 2
    ty, tcb, tcr = planes(frames[0], w, h)
    sy, sb, sr = ty.astype(np.uint32), tcb.astype(np.uint32), tcr.astype(np.uint32)
    cy = np.ones((h, w), np.uint32)
    cc = np.ones((ch, cw), np.uint32)
    accepted = 0
    for j in range(1, n):
        fy, fcb, fcr = planes(frames[j], w, h)
        for by in range(0, h, 16):
            bh = min(16, h - by)
            for bx in range(0, w, 16):
                bw = min(16, w - bx)
                sad = int(np.abs(ty[by:by + bh, bx:bx + bw].astype(np.int64)
                                 - fy[by:by + bh, bx:bx + bw].astype(np.int64)).sum())
                if sad > bw * bh * 6:
                    continue
                accepted += 1
                sy[by:by + bh, bx:bx + bw] += fy[by:by + bh, bx:bx + bw]
                cy[by:by + bh, bx:bx + bw] += 1
                cx0, cy0 = bx // 2, by // 2
                cx1, cy1 = min(cw, (bx + bw + 1) // 2), min(ch, (by + bh + 1) // 2)
                sb[cy0:cy1, cx0:cx1] += fcb[cy0:cy1, cx0:cx1]
                sr[cy0:cy1, cx0:cx1] += fcr[cy0:cy1, cx0:cx1]
                cc[cy0:cy1, cx0:cx1] += 1
    if accepted == 0:
        return None
    oy = ((sy + cy // 2) // cy).astype(np.uint8)
    ob = ((sb + cc // 2) // cc).astype(np.uint8)
    orr = ((sr + cc // 2) // cc).astype(np.uint8)
    return oy.tobytes() + ob.tobytes() + orr.tobytes()
