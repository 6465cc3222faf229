"""The env-gated component trace (append_hogbom_trace, lib.rs:54046-54066):
one JSON line per component with the reference's fields, appended only when
CASA_RS_HOGBOM_TRACE names a file (no GPU needed)."""
import json

import numpy as np

from casars_cuda import append_hogbom_trace


def test_trace_lines_follow_the_reference_fields(tmp_path, monkeypatch):
    path = tmp_path / "hogbom.jsonl"
    monkeypatch.setenv("CASA_RS_HOGBOM_TRACE", str(path))
    comps = np.array([[3, 5], [7, 1]], np.int32)
    peaks = np.array([1.5, -0.25], np.float32)
    fluxes = np.float32(0.1) * peaks
    assert append_hogbom_trace(comps, peaks, fluxes, reffreq_hz=1.4e9) == 2
    assert append_hogbom_trace(comps[:1], peaks[:1], fluxes[:1], reffreq_hz=1.4e9) == 1
    lines = [json.loads(x) for x in path.read_text().splitlines()]
    assert [x["cycle_update"] for x in lines] == [0, 1, 0]
    assert lines[1] == {"event": "component", "backend": "cuda", "reffreq_hz": 1.4e9,
                        "cycle_update": 1, "x": 7, "y": 1, "peak": float(np.float32(-0.25)),
                        "component": float(fluxes[1])}
    assert list(lines[0]) == ["event", "backend", "reffreq_hz", "cycle_update", "x", "y",
                              "peak", "component"]


def test_no_trace_without_the_variable(tmp_path, monkeypatch):
    monkeypatch.delenv("CASA_RS_HOGBOM_TRACE", raising=False)
    comps = np.array([[1, 2]], np.int32)
    assert append_hogbom_trace(comps, np.ones(1, np.float32), np.ones(1, np.float32)) == 0
    assert not list(tmp_path.iterdir())
