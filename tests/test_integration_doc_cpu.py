"""The cgo binding in the integration guide (the Go side a govid maintainer
adds for ebiv.Codec and the AsyncPlayer frame source) uses only names the
C-ABI headers declare: every C.<name> of its Go blocks is a function, type or
constant of include/*.h, and every C struct field it reads is a field there.
No Go toolchain is available, so this keeps the documented binding in step
with the headers."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CGO_BUILTINS = {"int", "int32_t", "int64_t", "uint8_t", "uint32_t", "uint64_t", "size_t", "double", "char",
                "GoString", "GoBytes", "CString", "free"}


def _go_blocks() -> list[str]:
    return re.findall(r"```go\n(.*?)```", (ROOT / "INTEGRATION.md").read_text(), re.S)


def _headers() -> str:
    return "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))


def test_every_c_name_of_the_binding_is_declared():
    blocks = _go_blocks()
    assert blocks, "the integration guide shows the Go binding"
    hdr = _headers()
    used = set()
    for b in blocks:
        used |= set(re.findall(r"\bC\.([A-Za-z_][A-Za-z0-9_]*)", b))
    missing = sorted(n for n in used - CGO_BUILTINS if not re.search(rf"\b{re.escape(n)}\b", hdr))
    assert not missing, f"not declared in include/*.h: {missing}"
    assert {"ebivgpu_decode", "ebivgpu_flush", "ebivgpu_source_next"} <= used


def test_every_struct_field_the_binding_reads_is_declared():
    hdr = _headers()
    fields = set()
    for b in _go_blocks():
        fields |= {f for f in re.findall(r"\.([a-z][a-z0-9]*_[a-z0-9_]+)\b", b)
                   if not f.startswith("ebivgpu_") and f not in CGO_BUILTINS}
    assert fields
    missing = sorted(f for f in fields if not re.search(rf"\b{re.escape(f)}\s*[;,\[]", hdr))
    assert not missing, f"struct fields not in include/*.h: {missing}"
