"""The Python mirror's stream handover, without a GPU.

Context.use_torch_stream passes torch's current stream to cr_ctx_set_stream.
Torch's default stream has the handle 0, which the library would take as
"the context's own (non-blocking) stream" -- not ordered with torch's work --
so the binding must pass it as cudaStreamLegacy (1), and any other stream
as its own handle.  The library call is replaced by a recorder here.
"""
import ctypes as C

import pytest

torch = pytest.importorskip("torch")

from casars_cuda import imaging  # noqa: E402


class _Stream:
    def __init__(self, handle):
        self.cuda_stream = handle


def _context():
    ctx = object.__new__(imaging.Context)
    ctx._h = C.c_void_p(0x1234)
    ctx.device = 0
    return ctx


@pytest.mark.parametrize("handle, passed", [(0, imaging.CUDA_STREAM_LEGACY), (0xBEEF, 0xBEEF)])
def test_torch_stream_handles(monkeypatch, handle, passed):
    seen = []
    monkeypatch.setattr(imaging, "call", lambda name, *args: seen.append((name, args)))
    monkeypatch.setattr(torch.cuda, "is_available", lambda: True)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda device=None: _Stream(handle))
    _context().use_torch_stream()
    assert len(seen) == 1
    name, args = seen[0]
    assert name == "cr_ctx_set_stream"
    assert args[1].value == passed


def test_own_stream_is_null(monkeypatch):
    seen = []
    monkeypatch.setattr(imaging, "call", lambda name, *args: seen.append((name, args)))
    _context().use_own_stream()
    assert len(seen) == 1 and seen[0][0] == "cr_ctx_set_stream" and seen[0][1][1] is None
