"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares."""
import ctypes as C
import re
from pathlib import Path

from govid_gb300 import _native

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(ebiv\w*)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(_native.LIB_PATH))
    names = _declared()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_device_probe_and_status_strings():
    L = _native.lib()
    assert L.ebivgpu_device_available() in (0, 1)
    assert L.ebivgpu_status_string(1) == b"ebiv: corrupt stream"


def test_struct_layouts_match_the_header():
    # The ctypes mirrors of the public structs have the C sizes (a field
    # added on one side only would shift every later field).
    L = _native.lib()
    sizes = (C.c_size_t * 5)()
    assert L.ebivgpu_abi_sizes(sizes, 5) == 5
    mirrors = [_native.Frame, _native.PlaneView, _native.ServeOptions, _native.ServeStats, _native.SourceFrame]
    assert [C.sizeof(m) for m in mirrors] == list(sizes)
