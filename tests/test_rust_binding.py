"""The Rust binding (bindings/rust/cassia-gb300-sys) against the C header.

No Rust toolchain is available to compile the crate, so this checks it as
text: every function of include/cassia_gb300.h is declared in the crate's
extern block with the same argument and return types, every struct has the
same fields in the same order with the same types, every status/enum
constant has the same value, and the dlopen wrapper's signatures agree with
the extern block.  A header change without the matching binding change fails
here.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cassia_gb300.h")
CRATE = os.path.join(ROOT, "bindings", "rust", "cassia-gb300-sys")
LIB_RS = os.path.join(CRATE, "src", "lib.rs")
DL_RS = os.path.join(CRATE, "src", "dl.rs")

C_TO_RUST = {
    "uint8_t": "u8", "uint32_t": "u32", "uint64_t": "u64", "int32_t": "i32", "int": "c_int", "float": "f32",
    "size_t": "usize", "char": "c_char", "void": "c_void",
}


def _c_header():
    s = open(HEADER).read()
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(CGB_\w+)\s+(\d+)u?\b", s)}
    s = re.sub(r"/\*.*?\*/", "", s, flags=re.S)
    funcs = {}
    for m in re.finditer(r"CGB_EXPORT\s+([^;(]*?)\s*\b(\w+)\s*\(([^;]*?)\)\s*;", s, flags=re.S):
        ret, name, params = " ".join(m.group(1).split()), m.group(2), " ".join(m.group(3).split())
        args = [] if params in ("void", "") else [p.strip() for p in params.split(",")]
        funcs[name] = ([_c_decl(a) for a in args], _c_type(ret.replace("*", " * ").split()))
    structs = {}
    for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", s, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            toks = re.findall(r"\w+|\*|\[\d+\]|,", decl)
            # "float a, b, c" declares several fields of one type
            first = toks.index(",") if "," in toks else len(toks)
            head, rest = toks[:first], toks[first:]
            fields.append(_c_field(head))
            base = [t for t in head[:-1] if not re.fullmatch(r"\[\d+\]", t)]
            while rest:
                rest = rest[1:]
                nxt = rest.index(",") if "," in rest else len(rest)
                fields.append(_c_field(base + rest[:nxt]))
                rest = rest[nxt:]
        structs[m.group(1)] = fields
    fn_ptr = re.search(r"typedef\s+void\s*\(\*\s*cgb_flush_fn\)\s*\(([^)]*)\)\s*;", s)
    flush = [_c_decl(a.strip()) for a in fn_ptr.group(1).split(",")]
    return funcs, structs, consts, flush


def _c_type(toks):
    """Rust spelling of a C type given as tokens without a name."""
    i = 0
    const = False
    base = None
    while i < len(toks) and toks[i] != "*":
        if toks[i] == "const":
            const = True
        else:
            base = toks[i]
        i += 1
    rust = C_TO_RUST.get(base, base)
    while i < len(toks):
        assert toks[i] == "*"
        rust = ("*const " if const else "*mut ") + rust
        i += 1
        const = i < len(toks) and toks[i] == "const"
        if const:
            i += 1
    return rust


def _c_decl(decl):
    """(name, Rust type) of a C parameter; `T name[N]` decays to a pointer."""
    toks = re.findall(r"\w+|\*|\[\d+\]", decl)
    if re.fullmatch(r"\[\d+\]", toks[-1]):
        return toks[-2], _c_type(toks[:-2] + ["*"])
    return toks[-1], _c_type(toks[:-1])


def _c_field(toks):
    if re.fullmatch(r"\[\d+\]", toks[-1]):
        return toks[-2], f"[{_c_type(toks[:-2])}; {toks[-1][1:-1]}]"
    return toks[-1], _c_type(toks[:-1])


def _split_args(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "(<[":
            depth += 1
        elif ch in ")>]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [a.strip() for a in out if a.strip()]


def _rust_args(s):
    res = []
    for a in _split_args(s):
        name, ty = a.split(":", 1)
        res.append((name.strip(), " ".join(ty.split())))
    return res


def _rust_lib():
    s = open(LIB_RS).read()
    s = re.sub(r"//[^\n]*", "", s)
    block = re.search(r'extern "C" \{(.*)\n\}', s, flags=re.S).group(1)
    funcs = {}
    for m in re.finditer(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        funcs[m.group(1)] = (_rust_args(m.group(2)), " ".join((m.group(3) or "()").split()))
    structs = {}
    for m in re.finditer(r"pub struct (\w+) \{(.*?)\n\}", s, flags=re.S):
        fields = []
        for line in m.group(2).split("\n"):
            line = line.strip().rstrip(",")
            if line.startswith("pub "):
                name, ty = line[4:].split(":", 1)
                fields.append((name.strip(), " ".join(ty.split())))
        structs[m.group(1)] = fields
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"pub const (CGB_\w+): \w+ = (\d+);", s)}
    flush = re.search(r'pub type cgb_flush_fn = Option<unsafe extern "C" fn\((.*?)\)>;', s, flags=re.S)
    return funcs, structs, consts, _rust_args(flush.group(1))


def test_every_function_declared_with_the_same_signature():
    cf, _, _, _ = _c_header()
    rf, _, _, _ = _rust_lib()
    assert set(cf) == set(rf), (sorted(set(cf) - set(rf)), sorted(set(rf) - set(cf)))
    for name, (cargs, cret) in cf.items():
        rargs, rret = rf[name]
        assert [t for _, t in rargs] == [t for _, t in cargs], (name, rargs, cargs)
        assert [n for n, _ in rargs] == [n for n, _ in cargs], (name, "argument names")
        assert rret == cret, (name, rret, cret)


def test_every_struct_has_the_same_fields_in_order():
    _, cs, _, cflush = _c_header()
    _, rs, _, rflush = _rust_lib()
    for name in ("cgb_props", "cgb_buffer", "cgb_rect", "cgb_stats", "cgb_tuning", "cgb_cassia_styling",
                 "cgb_layer_update"):
        assert name in cs and name in rs, name
        assert rs[name] == cs[name], (name, rs[name], cs[name])
    # the buffer's flusher callback: fields present and the callback's own signature
    assert [n for n, _ in cs["cgb_buffer"]][-2:] == ["flusher", "flusher_user"]
    assert rflush == cflush
    assert set(cs) <= set(rs)


def test_every_constant_has_the_same_value():
    _, _, cc, _ = _c_header()
    _, _, rc, _ = _rust_lib()
    assert cc, "no constants parsed from the header"
    assert cc == rc, ({k: (cc.get(k), rc.get(k)) for k in set(cc) | set(rc) if cc.get(k) != rc.get(k)})


def test_dlopen_wrapper_agrees_with_the_extern_block():
    rf, _, _, _ = _rust_lib()
    s = open(DL_RS).read()
    api = re.search(r"struct CassiaGb300Api \{(.*?)\n\}", s, flags=re.S).group(1)
    seen = 0
    for m in re.finditer(r'(\w+): unsafe extern "C" fn\((.*?)\)\s*(?:->\s*([^,]+))?,', api, flags=re.S):
        name, args, ret = m.group(1), _rust_args(m.group(2)), " ".join((m.group(3) or "()").split())
        want_args, want_ret = rf[name]
        norm = lambda t: t.replace("*mut cgb_composition", "*mut c_void")  # the opaque handle as a void pointer
        assert [norm(t) for _, t in args] == [norm(t) for _, t in want_args], name
        assert ret == want_ret, name
        seen += 1
    assert seen >= 3
    assert "cgb_cassia_render" in api


def test_crate_manifest_links_the_library():
    toml = open(os.path.join(CRATE, "Cargo.toml")).read()
    assert 'name = "cassia-gb300-sys"' in toml and 'links = "cassia_gb300"' in toml
    build = open(os.path.join(CRATE, "build.rs")).read()
    assert "rustc-link-lib=dylib=cassia_gb300" in build
