"""Generate src/sys.rs, the raw Rust declarations of include/casars_cuda.h.

The header is plain C with a narrow vocabulary (fixed-width integers,
float, double, char, void, opaque handle typedefs, typedef'd structs and
#define constants), so a small parser replaces bindgen, which the crate
would otherwise need at build time.  Run it after changing the header:

    python casa-rs_gb300/rust/casars-cuda-sys/gen_sys.py            # rewrite
    python casa-rs_gb300/rust/casars-cuda-sys/gen_sys.py --check    # exit 1 if stale
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.normpath(os.path.join(HERE, "..", "..", "..", "include", "casars_cuda.h"))
OUT = os.path.join(HERE, "src", "sys.rs")

SCALARS = {"int32_t": "i32", "int64_t": "i64", "uint8_t": "u8", "float": "f32",
           "double": "f64", "char": "c_char", "void": "c_void", "int": "c_int"}


def strip_comments(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def rust_type(ctype, opaque):
    """C type text (e.g. 'const float*', 'cr_ctx**') -> Rust type."""
    t = ctype.strip()
    stars = t.count("*")
    base = t.replace("*", " ").split()
    consts = [i for i, w in enumerate(base) if w == "const"]
    words = [w for w in base if w != "const"]
    if len(words) != 1:
        raise ValueError("unsupported C type: %r" % ctype)
    name = words[0]
    if name in SCALARS:
        r = SCALARS[name]
    elif name.startswith("cr_"):
        r = name
    else:
        raise ValueError("unsupported C type: %r" % ctype)
    if stars == 0:
        if r == "c_void":
            return None
        return r
    # 'const T*' -> *const T; 'T**' -> *mut *mut T ('const' only ever leads)
    lead_const = bool(consts) and consts[0] == 0
    for level in range(stars):
        innermost = level == 0
        r = ("*const " if (innermost and lead_const) else "*mut ") + r
    return r


def parse(text):
    src = strip_comments(text)
    consts = re.findall(r"^#define\s+(CR_\w+)\s+(-?\d+)", src, flags=re.M)
    opaque = re.findall(r"typedef\s+struct\s+(\w+)\s+\1\s*;", src)
    structs = []
    for body, name in re.findall(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"((?:const\s+)?\w+\s*\**)\s*(.*)$", decl)
            ctype, names = m.group(1), m.group(2)
            for nm in names.split(","):
                nm = nm.strip()
                extra = nm.count("*")
                fields.append((nm.replace("*", "").strip(), ctype + "*" * extra))
        structs.append((name, fields))
    funcs = []
    body = re.sub(r"typedef\s+struct\s*\{.*?\}\s*\w+\s*;", "", src, flags=re.S)
    body = re.sub(r"^#.*$", "", body, flags=re.M)
    for m in re.finditer(r"((?:const\s+)?\w+\s*\**)\s*(cr_\w+)\s*\(([^)]*)\)\s*;", body):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        params = []
        a = " ".join(args.split())
        if a and a != "void":
            for p in a.split(","):
                p = p.strip()
                pm = re.match(r"(.*?)(\w+)$", p)
                params.append((pm.group(2), pm.group(1)))
        funcs.append((name, ret, params))
    return consts, opaque, structs, funcs


RUST_KEYWORDS = {"type", "loop", "match", "ref", "move", "in", "fn", "mod", "use", "impl"}


def generate(text):
    consts, opaque, structs, funcs = parse(text)
    out = ["// Raw declarations of include/casars_cuda.h, written by gen_sys.py; do not edit.",
           "#![allow(non_camel_case_types)]", "",
           "use std::os::raw::{c_char, c_int, c_void};", ""]
    for name, value in consts:
        out.append("pub const %s: i32 = %s;" % (name, value))
    out.append("")
    for name in opaque:
        out.append("#[repr(C)]")
        out.append("pub struct %s {" % name)
        out.append("    _private: [u8; 0],")
        out.append("}")
        out.append("")
    for name, fields in structs:
        pod = all("*" not in c for _, c in fields)
        out.append("#[repr(C)]")
        out.append("#[derive(Clone, Copy, Debug%s)]" % (", Default" if pod else ""))
        out.append("pub struct %s {" % name)
        for fname, ctype in fields:
            out.append("    pub %s: %s," % (fname, rust_type(ctype, opaque)))
        out.append("}")
        out.append("")
    out.append('#[link(name = "casars_cuda")]')
    out.append('extern "C" {')
    for name, ret, params in funcs:
        ps = ", ".join("%s: %s" % (p + "_" if p in RUST_KEYWORDS else p, rust_type(t, opaque))
                       for p, t in params)
        r = rust_type(ret, opaque)
        out.append("    pub fn %s(%s)%s;" % (name, ps, "" if r is None else " -> " + r))
    out.append("}")
    return "\n".join(out) + "\n"


def main():
    text = open(HEADER).read()
    rs = generate(text)
    if "--check" in sys.argv[1:]:
        cur = open(OUT).read() if os.path.exists(OUT) else ""
        if cur != rs:
            print("src/sys.rs is stale: run gen_sys.py")
            return 1
        return 0
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    open(OUT, "w").write(rs)
    return 0


if __name__ == "__main__":
    sys.exit(main())
