"""The Rust binding crate (casa-rs_gb300/rust/casars-cuda-sys) against the C header.

No Rust toolchain is available to build the crate, so these checks keep it
honest by text: src/sys.rs is exactly what gen_sys.py makes from
include/casars_cuda.h; every header function is declared there with the
argument count and the scalar/pointer kinds of the ctypes binding the GPU
tests use; the #[repr(C)] structs list the ctypes structs' fields in order;
and every sys:: item the safe layer uses exists.
"""
import ctypes as C
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CRATE = os.path.join(ROOT, "casa-rs_gb300", "rust", "casars-cuda-sys")
sys.path.insert(0, os.path.join(ROOT, "casa-rs_gb300"))

from casars_cuda import _lib  # noqa: E402


def _sys_rs():
    return open(os.path.join(CRATE, "src", "sys.rs")).read()


def _rust_fns():
    out = {}
    for name, args, ret in re.findall(r"pub fn (cr_\w+)\((.*?)\)(?: -> ([^;]+))?;", _sys_rs()):
        params = [a.split(":", 1)[1].strip() for a in args.split(",") if a.strip()]
        out[name] = (params, ret or None)
    return out


def test_sys_rs_is_generated_from_the_header():
    r = subprocess.run([sys.executable, os.path.join(CRATE, "gen_sys.py"), "--check"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_every_header_function_matches_the_ctypes_binding():
    fns = _rust_fns()
    header = open(os.path.join(ROOT, "include", "casars_cuda.h")).read()
    declared = set(re.findall(r"\b(cr_\w+)\s*\(", re.sub(r"/\*.*?\*/", "", header, flags=re.S)))
    assert declared == set(fns)
    assert set(_lib.SIGNATURES) <= set(fns)
    ints = {C.c_int32: "i32", C.c_int64: "i64", C.c_float: "f32", C.c_double: "f64",
            C.c_int: "c_int"}
    for name, (restype, argtypes) in _lib.SIGNATURES.items():
        params, ret = fns[name]
        assert len(params) == len(argtypes), name
        for rs, ct in zip(params, argtypes):
            if rs.startswith("*"):
                assert ct not in ints, (name, rs, ct)
            else:
                assert ints.get(ct) == rs or (rs == "i32" and ct is C.c_int), (name, rs, ct)
        if restype is None:
            assert ret is None, name
        elif restype in ints:
            assert ret in (ints[restype], "c_int", "i32"), (name, ret)
        else:
            assert ret is not None and ret.startswith("*"), (name, ret)


def test_structs_match_the_ctypes_layout():
    rs = _sys_rs()
    structs = dict(re.findall(r"pub struct (cr_\w+) \{\n(.*?)\n\}", rs, flags=re.S))
    pairs = {"cr_geometry": _lib.Geometry, "cr_grid_info": _lib.GridInfo,
             "cr_wproj_info": _lib.WProjInfo, "cr_vis_batch": _lib.VisBatch,
             "cr_cube_batch": _lib.CubeBatch, "cr_row_runs": _lib.RowRuns,
             "cr_polarization": _lib.Polarization, "cr_beam": _lib.Beam,
             "cr_sums": _lib.Sums, "cr_psf_state": _lib.PsfState, "cr_timings": _lib.Timings,
             "cr_row_feed_config": _lib.RowFeedConfig, "cr_row_block": _lib.RowBlock,
             "cr_row_feed_summary": _lib.RowFeedSummary}
    sizes = {"i32": 4, "i64": 8, "f32": 4, "f64": 8, "u8": 1}
    for name, cls in pairs.items():
        fields = re.findall(r"pub (\w+): ([^,]+),", structs[name])
        assert [f for f, _ in fields] == [f for f, _ in cls._fields_], name
        for (f, t), (_, ct) in zip(fields, cls._fields_):
            if t in pairs:   # a nested struct
                assert C.sizeof(ct) == C.sizeof(pairs[t]), (name, f, t)
                continue
            want = 8 if t.startswith("*") else sizes[t]
            assert C.sizeof(ct) == want, (name, f, t)


def test_safe_layer_uses_declared_items_only():
    fns = _rust_fns()
    consts = set(re.findall(r"pub const (CR_\w+):", _sys_rs()))
    types = set(re.findall(r"pub struct (cr_\w+)", _sys_rs()))
    for fname in ("lib.rs", "backend.rs"):
        src = open(os.path.join(CRATE, "src", fname)).read()
        for item in set(re.findall(r"sys::(\w+)", src)):
            assert item in fns or item in consts or item in types, (fname, item)
    lib = open(os.path.join(CRATE, "src", "lib.rs")).read()
    assert "pub mod sys;" in lib and "pub mod backend;" in lib
