"""The Rust crate's raw bindings (prestige_gb300/rust/prestige_gpu/src/ffi.rs) against the C
header: every entry point of include/prestige_gpu.h is declared with the same number of
parameters, and the three structs list the same fields in the same order, with array lengths.
No Rust toolchain is needed (nor present on these machines): this reads both files as text."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "prestige_gpu.h")
FFI = os.path.join(ROOT, "prestige_gb300", "rust", "prestige_gpu", "src", "ffi.rs")


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", " ", s, flags=re.S)


def _header_functions():
    src = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"\b(?:int|void|const char\s*\*)\s+(pg_\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def _rust_functions():
    src = open(FFI).read()
    out = {}
    for m in re.finditer(r"pub fn (pg_\w+)\s*\(([^)]*)\)", src, flags=re.S):
        args = m.group(2).strip().rstrip(",")
        out[m.group(1)] = 0 if not args else args.count(",") + 1
    return out


def _c_struct(name):
    src = _strip_c_comments(open(HEADER).read())
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        names = decl.split(None, 1)[1] if not decl.startswith("long long") else decl[len("long long"):]
        for part in names.split(","):
            part = part.strip()
            m = re.match(r"(\w+)(?:\[(\d+)\])?", part)
            fields.append((m.group(1), int(m.group(2)) if m.group(2) else 0))
    return fields


def _rust_struct(name):
    src = open(FFI).read()
    body = re.search(r"pub struct %s \{(.*?)\n\}" % name, src, flags=re.S).group(1)
    fields = []
    for m in re.finditer(r"pub (\w+): (\[[^\]]*\]|\w+)", body):
        arr = re.match(r"\[\w+; (\d+)\]", m.group(2))
        fields.append((m.group(1), int(arr.group(1)) if arr else 0))
    return fields


def test_every_entry_point_is_bound_with_its_arity():
    c = _header_functions()
    r = _rust_functions()
    assert len(c) >= 35
    assert set(c) == set(r), (sorted(set(c) - set(r)), sorted(set(r) - set(c)))
    for name, arity in c.items():
        assert r[name] == arity, (name, arity, r[name])


def test_structs_have_the_header_layout():
    for name in ("pg_config", "pg_info", "pg_timing"):
        assert _rust_struct(name) == _c_struct(name), name


def test_status_and_enum_values_match():
    hdr = _strip_c_comments(open(HEADER).read())
    ffi = open(FFI).read()
    for m in re.finditer(r"\b(PG_[A-Z0-9_]+)\s*=\s*(\d+)", hdr):
        rm = re.search(r"pub const %s: c_int = (\d+);" % m.group(1), ffi)
        assert rm and rm.group(1) == m.group(2), m.group(1)
