"""Committed fixtures (tests/golden/, generated by make_golden.py): the
encoder regenerates them byte for byte on this host, and the CPU oracle's
per-frame decode hashes match the recorded ones."""
import hashlib
import json
from pathlib import Path

import pytest

import ebiv_oracle
from govid_gb300 import ebiv

GOLDEN = Path(__file__).resolve().parent / "golden"
SPEC = json.loads((GOLDEN / "golden.json").read_text())


def _h(b):
    return hashlib.sha256(b).hexdigest()


@pytest.mark.parametrize("name", sorted(SPEC))
def test_encoder_regenerates_fixture(name):
    import sys

    sys.path.insert(0, str(GOLDEN))
    import make_golden

    w, h, build = make_golden.fixtures()[name]
    assert _h(build()) == SPEC[name]["sha256"]


@pytest.mark.parametrize("name", sorted(SPEC))
def test_oracle_decodes_fixture(name):
    data = (GOLDEN / f"{name}.ebiv").read_bytes()
    assert _h(data) == SPEC[name]["sha256"]
    pk = [p.data for p in ebiv.Reader(data).packets()]
    got = ebiv_oracle.decode_all(pk)
    for i, ((st, planes), want) in enumerate(zip(got, SPEC[name]["frames"])):
        assert st == want["status"], f"{name} frame {i}"
        assert (_h(planes) if planes else None) == want["sha256"], f"{name} frame {i}"
