"""The Rust binding a maintainer of the crate would add (the complete `extern "C"` block in
the integration guide) agrees with include/split_operator.h: every declared entry point
appears once, with the same parameter names, the same order and the mapped types, and every
SO_* constant has the header's value.  Text only: no Rust toolchain, no GPU."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HANDLES = {"so_grid", "so_wave_function", "so_operator", "so_operation_stack", "so_propagation",
           "so_batch", "so_mlp"}
SCALARS = {"char": "c_char", "int": "c_int", "double": "f64", "float": "f32", "uint64_t": "u64",
           "size_t": "usize", "void": "c_void", "so_time_grid": "SoTimeGrid"}
RUST_KEYWORDS = {"in", "type", "ref", "fn", "move", "loop", "match", "box", "use", "mod", "self"}


def rust_type(c):
    """C type text -> Rust type text: the pointee of each '*' is const when a 'const'
    precedes it (on the base type for the first level, after the previous '*' otherwise)."""
    m = re.fullmatch(r"(const )?(\w+)((?:\s*\*\s*(?:const)?)*)", " ".join(c.split()))
    assert m, c
    base_const, base, stars = m.group(1), m.group(2), re.findall(r"\*\s*(const)?", m.group(3))
    t = SCALARS.get(base) or (base if base in HANDLES else None)
    assert t, c
    quals = [bool(base_const)] + [bool(q) for q in stars[:-1]]
    for i in range(len(stars)):
        t = ("*const " if quals[i] else "*mut ") + t
    return t


def header_decls():
    src = open(os.path.join(ROOT, "include", "split_operator.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#[^\n]*", "", src)
    out = {}
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(so_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        params = []
        for a in args.split(","):
            a = " ".join(a.split())
            if not a or a == "void":
                continue
            m = re.fullmatch(r"(.*?)(\w+)", a)
            pname = m.group(2) + ("_" if m.group(2) in RUST_KEYWORDS else "")
            params.append((pname, rust_type(m.group(1).strip())))
        ret = " ".join(ret.split())
        assert name not in out, name
        out[name] = (params, None if ret == "void" else rust_type(ret))
    return out, dict((k, int(v)) for k, v in re.findall(r"\b(SO_[A-Z0-9_]+)\s*=\s*(\d+)", src))


def rust_block():
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = doc.split("### The complete `extern` block", 1)[1]
    code = re.search(r"```rust\n(.*?)```", sec, flags=re.S).group(1)
    fns = {}
    ext = code.split('extern "C" {', 1)[1]
    for name, args, ret in re.findall(r"pub fn (\w+)\((.*?)\)(?:\s*->\s*([^;]+?))?\s*;", ext, flags=re.S):
        params = []
        for a in args.split(","):
            a = " ".join(a.split())
            if a:
                pname, ptype = a.split(":", 1)
                params.append((pname.strip(), ptype.strip()))
        assert name not in fns, name
        fns[name] = (params, ret.strip() if ret else None)
    consts = {k: int(v) for k, v in re.findall(r"pub const (SO_[A-Z0-9_]+): c_int = (\d+);", code)}
    return fns, consts, code


def test_every_header_declaration_is_bound_with_mapped_types():
    decls, _ = header_decls()
    fns, _, _ = rust_block()
    assert len(decls) > 100
    assert sorted(decls) == sorted(fns), (sorted(set(decls) ^ set(fns)))
    wrong = [n for n in decls if decls[n] != fns[n]]
    assert not wrong, [(n, decls[n], fns[n]) for n in wrong]


def test_constants_and_types_match_the_header():
    _, hconsts = header_decls()
    _, rconsts, code = rust_block()
    assert hconsts and hconsts == rconsts
    for h in HANDLES:
        assert re.search(rf"pub type {h} = \*mut {h}_t;", code), h
    # so_time_grid: double step, uint64_t step_no, int im_time, in this order
    assert "pub struct SoTimeGrid { pub step: f64, pub step_no: u64, pub im_time: c_int }" in code


def test_type_mapping_rules():
    assert rust_type("const double* const*") == "*const *const f64"
    assert rust_type("double* const*") == "*const *mut f64"
    assert rust_type("const so_grid*") == "*const so_grid"
    assert rust_type("so_propagation*") == "*mut so_propagation"
    assert rust_type("void*") == "*mut c_void"
    assert rust_type("size_t") == "usize"
