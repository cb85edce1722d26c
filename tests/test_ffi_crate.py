"""The Rust binding crate (physics-sim_gb300/ffi) against include/dem.h.

No Rust toolchain exists here, so the crate is checked by reading it: every
struct of the header has a #[repr(C)] struct in src/lib.rs with the same
fields in the same order and the same C types, and every function the
header declares is in the crate's extern "C" block with the same parameter
and return types.  A field added to the header and not to the crate (or the
other way round) fails here.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dem.h")
CRATE = os.path.join(ROOT, "physics-sim_gb300", "ffi")

SCALARS = {"int32_t": "i32", "int": "c_int", "float": "f32", "double": "f64", "int64_t": "i64",
           "char": "c_char", "void": "c_void", "uint32_t": "u32"}


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def _c_type(decl):
    """Rust spelling of one C declaration `type name` or `type name[N]`
    (struct field: arrays stay arrays)."""
    decl = " ".join(decl.split())
    m = re.match(r"^(.*?)(\w+)\s*(\[(\w+)\])?$", decl)
    base, name, arr = m.group(1).strip(), m.group(2), m.group(4)
    return name, _ptr_type(base, arr)


def _ptr_type(base, arr=None, param=False):
    # split "const T *const *" into the base type and the pointer levels
    toks = base.replace("*", " * ").split()
    quals, levels, cur_const = [], [], False
    core = None
    for t in toks:
        if t == "const":
            if core is None:
                quals.append("const")
            else:
                cur_const = True
                if levels:
                    levels[-1] = True
        elif t == "*":
            levels.append(False)
        else:
            core = t
    core_r = SCALARS.get(core, core)
    # innermost pointer's constness comes from the qualifier on the base type
    ty = core_r
    inner_const = "const" in quals
    for k, lvl_const in enumerate(levels):
        c = inner_const if k == 0 else levels[k - 1]
        ty = ("*const " if c else "*mut ") + ty
    if arr is not None:
        if param:
            ty = ("*const " if inner_const else "*mut ") + ty
        else:
            ty = "[%s; %s]" % (ty, arr)
    return ty


def header_structs():
    h = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} (\w+);", h, flags=re.S):
        fields = []
        for line in m.group(2).split(";"):
            line = " ".join(line.split())
            if not line:
                continue
            parts = [x.strip() for x in line.split(",")]
            name, ty = _c_type(parts[0])
            fields.append((name, ty))
            base = parts[0][:parts[0].rindex(name)]
            for extra in parts[1:]:       # int64_t a, b, c;
                fields.append(_c_type(base + extra))
        out[m.group(1)] = fields
    return out


def header_functions():
    h = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"^\s*([A-Za-z_][\w\s\*]*?)\b(dem_\w+)\s*\(([^;]*?)\)\s*;", h, flags=re.M):
        ret = m.group(1).strip()
        params = []
        args = " ".join(m.group(3).split())
        if args != "void":
            for a in args.split(","):
                a = a.strip()
                mm = re.match(r"^(.*?)(\w+)\s*(\[(\w+)\])?$", a)
                params.append(_ptr_type(mm.group(1), mm.group(4), param=True))
        out[m.group(2)] = (_ret_type(ret), params)
    return out


def _ret_type(ret):
    ret = " ".join(ret.split())
    if ret == "void":
        return None
    return _ptr_type(ret)


def crate_structs():
    src = open(os.path.join(CRATE, "src", "lib.rs")).read()
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\]\s*(?:#\[derive\([^)]*\)\]\s*)?pub struct (\w+) \{(.*?)\n\}", src, flags=re.S):
        fields = []
        for line in m.group(2).split(",\n"):
            line = line.strip().rstrip(",")
            mm = re.match(r"^pub (\w+): (.+)$", line)
            if mm:
                fields.append((mm.group(1), " ".join(mm.group(2).split())))
        out[m.group(1)] = fields
    return out


def crate_functions():
    src = open(os.path.join(CRATE, "src", "lib.rs")).read()
    block = src[src.index('extern "C" {'):]
    block = block[:block.index("\n}\n")]
    out = {}
    for m in re.finditer(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        params = []
        args = " ".join(m.group(2).split())
        if args:
            for a in args.split(","):
                a = a.strip()
                if a:
                    params.append(" ".join(a.split(":", 1)[1].split()))
        ret = " ".join(m.group(3).split()) if m.group(3) else None
        out[m.group(1)] = (ret, params)
    return out


def test_crate_files_exist():
    for f in ("Cargo.toml", "build.rs", os.path.join("src", "lib.rs")):
        assert os.path.exists(os.path.join(CRATE, f)), f
    toml = open(os.path.join(CRATE, "Cargo.toml")).read()
    assert 'links = "demgb"' in toml
    assert "rustc-link-lib=dylib=demgb" in open(os.path.join(CRATE, "build.rs")).read()


def test_every_header_struct_has_the_same_fields_in_the_crate():
    hs, cs = header_structs(), crate_structs()
    assert len(hs) >= 9
    for name, fields in hs.items():
        assert name in cs, "struct %s missing from the crate" % name
        assert cs[name] == fields, "struct %s differs:\n header %s\n crate  %s" % (name, fields, cs[name])


def test_every_header_function_is_bound_with_the_same_types():
    hf, cf = header_functions(), crate_functions()
    assert len(hf) >= 50
    for name, (ret, params) in hf.items():
        assert name in cf, "function %s missing from the crate's extern block" % name
        cret, cparams = cf[name]
        assert cret == ret, "%s returns %s in the header, %s in the crate" % (name, ret, cret)
        assert cparams == params, "%s parameters differ:\n header %s\n crate  %s" % (name, params, cparams)
    assert set(cf) <= set(hf), "crate binds functions the header does not declare: %s" % (set(cf) - set(hf))
