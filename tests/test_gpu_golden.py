"""GPU decode of the committed fixtures matches the recorded hashes, through
the C-ABI codec (per packet) and the batched engine (all fixtures at once)."""
import hashlib
import json
from pathlib import Path

import pytest

from govid_gb300 import ebiv

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
SPEC = json.loads((GOLDEN / "golden.json").read_text())


def _h(b):
    return hashlib.sha256(b).hexdigest()


@pytest.mark.parametrize("name", sorted(SPEC))
def test_codec_decodes_fixture(gpu_required, name):
    pk = [p.data for p in ebiv.Reader((GOLDEN / f"{name}.ebiv").read_bytes()).packets()]
    c = ebiv.Codec()
    for i, (p, want) in enumerate(zip(pk, SPEC[name]["frames"])):
        assert _h(c.decode(p).packed()) == want["sha256"], f"{name} frame {i}"


def test_batch_decodes_all_fixtures(gpu_required):
    b = ebiv.Batch(lookahead=3)
    ids = {}
    for name in sorted(SPEC):
        pk = [p.data for p in ebiv.Reader((GOLDEN / f"{name}.ebiv").read_bytes()).packets()]
        ids[b.add_stream(pk)] = name
    seen = 0
    while True:
        res = b.round()
        if not res:
            break
        for r in res:
            name = ids[r.stream]
            want = SPEC[name]["frames"][r.frame_index]
            assert r.status == want["status"]
            got = b.download(r, SPEC[name]["width"], SPEC[name]["height"])
            assert _h(got) == want["sha256"], f"{name} frame {r.frame_index}"
            seen += 1
    assert seen == sum(len(v["frames"]) for v in SPEC.values())
