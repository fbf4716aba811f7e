"""The Rust binding (rust/src/gb300.rs) against the C header (include/film_grain_gb300.h).

No Rust toolchain is needed: both files are parsed and compared -- every entry point, its argument
names, order and types, its return type, every struct's fields in order with their types, and every
constant -- so the crate-side binding cannot drift from the library's ABI.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "film_grain_gb300.h")
RUST = os.path.join(ROOT, "rust", "src", "gb300.rs")

SCALARS = {"int32_t": "i32", "uint32_t": "u32", "int64_t": "i64", "uint64_t": "u64", "float": "f32",
           "double": "f64", "size_t": "usize", "void": "c_void", "char": "c_char", "uint8_t": "u8",
           "unsigned long long": "u64", "fg_status": "i32", "int": "i32"}
RUST_KEYWORDS = {"in": "input"}


def _camel(name):
    return "".join(part.capitalize() for part in name.split("_"))


def _strip_c_comments(src):
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", " ", src)


def _rust_type(ctype, array=False):
    """C declaration type -> the Rust FFI type the binding must use."""
    t = " ".join(ctype.replace("volatile", " ").split())
    stars = t.count("*") + (1 if array else 0)
    t = t.replace("*", " ").strip()
    const = t.startswith("const ")
    base = t[6:].strip() if const else t
    base = SCALARS.get(base, _camel(base) if base.startswith("fg_") else base)
    if stars == 0:
        return base
    out = base
    for level in range(stars):
        innermost = level == 0
        out = ("*const " if (innermost and const) else "*mut ") + out
    return out


def _split_decl(decl):
    """'const float *lambda' -> ('const float *', 'lambda'); handles 'unsigned long long out[4]'."""
    decl = " ".join(decl.split())
    m = re.match(r"^(.*?)([A-Za-z_]\w*)\s*(\[\d*\])?$", decl)
    assert m, decl
    return m.group(1).strip(), m.group(2), bool(m.group(3))


def parse_header():
    src = _strip_c_comments(open(HEADER).read())
    structs, opaque, funcs, consts = {}, set(), {}, {}
    for name, body in re.findall(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*\w+\s*;", src, flags=re.S):
        fields = []
        for stmt in body.split(";"):
            stmt = " ".join(stmt.split())
            if not stmt:
                continue
            first, *rest = stmt.split(",")
            ctype, fname, arr = _split_decl(first)
            base = ctype.replace("*", "").strip()
            fields.append((fname, _rust_type(ctype, arr)))
            for extra in rest:  # 'uint32_t roi_x0, roi_y0' -> same base type
                stars = extra.count("*")
                fields.append((extra.replace("*", "").strip(), _rust_type(base + " *" * stars)))
        structs[_camel(name)] = fields
    for name in re.findall(r"typedef\s+struct\s+(\w+)\s+\w+\s*;", src):
        opaque.add(_camel(name))
    for ret, name, args in re.findall(r"FG_API\s+([\w\s\*]+?)\s*\b(fg_\w+)\s*\(([^)]*)\)\s*;", src, flags=re.S):
        params = []
        args = " ".join(args.split())
        if args and args != "void":
            for a in args.split(","):
                ctype, pname, arr = _split_decl(a)
                params.append((RUST_KEYWORDS.get(pname, pname), _rust_type(ctype, arr)))
        r = _rust_type(ret.strip())
        funcs[name] = (params, None if r == "c_void" else r)
    for body in re.findall(r"enum\s*\w*\s*\{(.*?)\}", src, flags=re.S):
        for k, v in re.findall(r"(FG_\w+)\s*=\s*(\d+)", body):
            consts[k] = int(v)
    for k, v in re.findall(r"#define\s+(FG_\w+)\s+\(?([\du\s\*]+)\)?\s*\n", src):
        consts[k] = eval(v.replace("u", ""))
    return structs, opaque, funcs, consts


def parse_rust():
    src = re.sub(r"//[^\n]*", " ", open(RUST).read())
    structs, opaque, funcs, consts = {}, set(), {}, {}
    for name, body in re.findall(r"#\[repr\(C\)\][^{;]*?pub\s+struct\s+(\w+)\s*\{(.*?)\}", src, flags=re.S):
        structs[name] = [(f, " ".join(t.split())) for f, t in re.findall(r"pub\s+(\w+)\s*:\s*([^,]+),", body)]
    opaque.update(re.findall(r"pub\s+enum\s+(\w+)\s*\{\s*\}", src))
    block = re.search(r'extern\s+"C"\s*\{(.*)\}', src, flags=re.S).group(1)
    for name, args, ret in re.findall(r"pub\s+fn\s+(\w+)\s*\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        params = []
        args = " ".join(args.split())
        if args:
            for a in args.split(","):
                a = a.strip()
                if a:
                    pname, ptype = a.split(":", 1)
                    params.append((pname.strip(), " ".join(ptype.split())))
        funcs[name] = (params, " ".join(ret.split()) if ret else None)
    for k, v in re.findall(r"pub\s+const\s+(FG_\w+)\s*:\s*\w+\s*=\s*([^;]+);", src):
        consts[k] = eval(v.replace("_", ""))
    return structs, opaque, funcs, consts


def test_rust_binding_has_every_entry_point_with_the_header_signature():
    _, _, cf, _ = parse_header()
    _, _, rf, _ = parse_rust()
    assert len(cf) >= 30
    assert set(cf) == set(rf), f"missing in Rust: {set(cf) - set(rf)}; extra: {set(rf) - set(cf)}"
    for name, (params, ret) in cf.items():
        assert rf[name] == (params, ret), f"{name}: header {params} -> {ret}; rust {rf[name]}"


def test_rust_structs_match_the_header_layout():
    cs, co, _, _ = parse_header()
    rs, ro, _, _ = parse_rust()
    assert set(cs) == set(rs), f"{set(cs) ^ set(rs)}"
    for name, fields in cs.items():
        assert rs[name] == fields, f"{name}: header {fields}\nrust {rs[name]}"
    assert co == ro == {"FgBatch"}


def test_rust_constants_match_the_header():
    _, _, _, cc = parse_header()
    _, _, _, rc = parse_rust()
    assert cc and set(cc) == set(rc), f"{set(cc) ^ set(rc)}"
    for k, v in cc.items():
        assert rc[k] == v, k


def test_safe_wrappers_call_the_declared_entry_points():
    """gb300_render.rs converts Params/Derived and calls the integrators through the binding."""
    src = open(os.path.join(ROOT, "rust", "src", "gb300_render.rs")).read()
    for fn in ("fg_render_pixelwise", "fg_render_grainwise", "fg_last_error_message"):
        assert f"ffi::{fn}(" in src
    _, _, rf, _ = parse_rust()
    rs, _, _, _ = parse_rust()
    # every FgParams / FgDerived field is set by the converters
    for struct, conv in (("FgParams", "to_fg_params"), ("FgDerived", "to_fg_derived")):
        body = src[src.index(f"pub fn {conv}"):]
        body = body[:body.index("\n}\n")]
        for field, _ in rs[struct]:
            assert re.search(rf"\b{field}\b", body), f"{conv} does not set {field}"
