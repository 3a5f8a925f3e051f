"""The three descriptions of the C ABI agree (CPU only, no GPU call):

* include/jump_mpm.h, compiled by gcc: offsetof/sizeof of every struct field;
* the ctypes mirror jump_gb300/_capi.py: the same field names at the same offsets;
* the Julia binding jump_gb300/julia/JumpGPU.jl (Julia is not installed here):
  its structs are parsed and laid out with C's rules (the layout Julia gives an
  isbits struct), and must have the header's field names, types and offsets;
  its ABI constant must be the header's; and every ccall's return and argument
  types must be those of the C prototype it calls.

A change to the header that is not mirrored in both bindings fails here."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

from jump_gb300 import _capi

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "jump_mpm.h")
JULIA = os.path.join(ROOT, "jump_gb300", "julia", "JumpGPU.jl")

JL_TO_C = {"MaterialDesc": "mpm_material_desc", "GridDesc": "mpm_grid_desc", "BodyDesc": "mpm_body_desc",
           "BodyView": "mpm_body_view", "Params": "mpm_params", "InstanceDesc": "mpm_instance_desc"}
CT_OF = {"mpm_material_desc": _capi.MaterialDesc, "mpm_grid_desc": _capi.GridDesc, "mpm_body_desc": _capi.BodyDesc,
         "mpm_body_view": _capi.BodyView, "mpm_params": _capi.Params, "mpm_instance_desc": _capi.InstanceDesc}


def _strip_c_comments(txt):
    return re.sub(r"/\*.*?\*/", "", txt, flags=re.S)


def c_structs():
    """{struct: [(field, ctype, count)]} from the header, in declaration order."""
    txt = _strip_c_comments(open(HEADER).read())
    out = {}
    for name, body, name2 in re.findall(r"typedef struct (\w+) \{(.*?)\} (\w+);", txt, flags=re.S):
        assert name == name2
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"((?:const )?[\w]+\s*\**)\s*(.*)$", decl)
            ctype = m.group(1).replace(" ", "")
            for item in m.group(2).split(","):
                item = item.strip()
                stars = len(item) - len(item.lstrip("*"))
                item = item.lstrip("*")
                mm = re.match(r"(\w+)(?:\[(\d+)\])?$", item)
                fields.append((mm.group(1), ctype + "*" * stars, int(mm.group(2) or 1)))
        out[name] = fields
    return out


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    """offset and size of every field, as gcc lays the header out"""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = c_structs()
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for s, fields in structs.items():
        lines.append(f'printf("%s %zu\\n", "{s}", sizeof({s}));')
        for f, _, _ in fields:
            lines.append(f'printf("%s.%s %zu %zu\\n", "{s}", "{f}", offsetof({s}, {f}), sizeof((({s}*)0)->{f}));')
    lines.append("return 0; }")
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines))
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True, capture_output=True)
    res = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        parts = line.split()
        res[parts[0]] = tuple(int(x) for x in parts[1:])
    return structs, res


def test_ctypes_mirror_matches_header(c_layout):
    structs, lay = c_layout
    assert set(CT_OF) == set(structs)
    for s, fields in structs.items():
        ct = CT_OF[s]
        assert [f for f, _ in ct._fields_] == [f for f, _, _ in fields], s
        assert C.sizeof(ct) == lay[s][0], s
        for f, _, _ in fields:
            off, size = lay[f"{s}.{f}"]
            assert getattr(ct, f).offset == off and getattr(ct, f).size == size, (s, f)


# ---------------------------------------------------------------------------
# the Julia binding

JL_SCALARS = {"Int32": ("int32_t", 4), "Int64": ("int64_t", 8), "Float64": ("double", 8)}


def julia_text():
    return re.sub(r"#.*", "", open(JULIA).read())


def julia_structs():
    out = {}
    for name, body in re.findall(r"^struct (\w+)\n(.*?)^end", julia_text(), flags=re.S | re.M):
        fields = []
        for line in body.splitlines():
            line = line.strip()
            if line:
                f, t = line.split("::")
                fields.append((f.strip(), t.strip()))
        out[name] = fields
    return out


def jl_type_info(t, structs):
    """(C type name, element count, size, alignment) of a Julia field type"""
    m = re.match(r"NTuple\{(\d+),(\w+)\}$", t)
    if m:
        ct, sz = JL_SCALARS[m.group(2)]
        return ct, int(m.group(1)), sz * int(m.group(1)), sz
    if t in JL_SCALARS:
        ct, sz = JL_SCALARS[t]
        return ct, 1, sz, sz
    m = re.match(r"Ptr\{(\w+)\}$", t)
    if m:
        inner = m.group(1)
        ct = JL_SCALARS[inner][0] if inner in JL_SCALARS else JL_TO_C[inner]
        return ct + "*", 1, 8, 8
    if t in structs:  # nested struct by value
        size, align = jl_layout(t, structs)[1:]
        return JL_TO_C[t], 1, size, align
    raise AssertionError(f"unmapped Julia field type {t}")


def jl_layout(name, structs):
    """({field: offset}, size, alignment) with C's layout rules"""
    off, align, offs = 0, 1, {}
    for f, t in structs[name]:
        _, _, size, a = jl_type_info(t, structs)
        off = (off + a - 1) // a * a
        offs[f] = off
        off += size
        align = max(align, a)
    return offs, (off + align - 1) // align * align, align


def test_julia_structs_match_header(c_layout):
    cstructs, lay = c_layout
    js = julia_structs()
    assert set(JL_TO_C) == set(js), "the binding declares one struct per header struct"
    for jn, fields in js.items():
        cn = JL_TO_C[jn]
        cf = cstructs[cn]
        assert [f for f, _ in fields] == [f for f, _, _ in cf], jn
        offs, size, _ = jl_layout(jn, js)
        assert size == lay[cn][0], (jn, size, lay[cn][0])
        for (f, t), (_, ctype, count) in zip(fields, cf):
            assert offs[f] == lay[f"{cn}.{f}"][0], (jn, f)
            jct, jcount, _, _ = jl_type_info(t, js)
            assert jct == ctype.replace("const", "") and jcount == count, (jn, f, t, ctype, count)


def test_julia_abi_version_matches_header():
    hdr = int(re.search(r"#define JUMP_MPM_ABI_VERSION (\d+)", open(HEADER).read()).group(1))
    jl = int(re.search(r"const ABI = (\d+)", open(JULIA).read()).group(1))
    assert jl == hdr == _capi.ABI_VERSION


def c_prototypes():
    """{symbol: (return type, [argument types])}, normalised"""
    txt = _strip_c_comments(open(HEADER).read())
    out = {}
    for ret, name, args in re.findall(r"^\s*(?:const\s+)?(\w+\s*\**)\s*(mpm_\w+)\(([^)]*)\);", txt,
                                      flags=re.M | re.S):
        types = []
        for a in args.split(","):
            a = " ".join(a.split())
            if not a or a == "void":
                continue
            a = re.sub(r"\bconst\b", "", a).strip()
            m = re.match(r"(\w+)\s*(\**)\s*\w+$", a)
            types.append(_canon_c(m.group(1), len(m.group(2))))
        out[name] = (_canon_c(ret.replace("*", "").strip(), ret.count("*")), types)
    return out


C_BASE = {"int": "i32", "int32_t": "i32", "int64_t": "i64", "double": "f64", "size_t": "usize", "char": "char",
          "void": "void", "mpm_ctx": "void", "mpm_batch": "void"}


def _canon_c(base, stars):
    b = C_BASE.get(base, base)
    if b == "char" and stars == 1:
        return "cstring"
    return b + "*" * stars


JL_BASE = {"Cint": "i32", "Int32": "i32", "Int64": "i64", "Float64": "f64", "Csize_t": "usize", "Cvoid": "void",
           "Cstring": "cstring"}


def _canon_jl(t):
    t = t.strip()
    m = re.match(r"(?:Ptr|Ref)\{(.*)\}$", t)
    if m:
        return _canon_jl(m.group(1)) + "*"
    if t in JL_BASE:
        return JL_BASE[t]
    return JL_TO_C[t]


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({":
            depth += 1
        elif ch in ")}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur)
    return [p.strip() for p in parts]


def julia_ccalls():
    """[(symbol, return type, [argument types])] of every ccall in the binding"""
    txt = julia_text()
    out = []
    for m in re.finditer(r"ccall\(\(:(\w+), lib\),", txt):
        i = m.end()
        depth, j = 1, i
        while depth:  # to the ccall's closing parenthesis
            depth += {"(": 1, ")": -1}.get(txt[j], 0)
            j += 1
        args = _split_top(txt[i:j - 1])
        ret, tup = args[0], args[1]
        assert tup.startswith("(") and tup.endswith(")"), (m.group(1), tup)
        types = [_canon_jl(t) for t in _split_top(tup[1:-1])]
        out.append((m.group(1), _canon_jl(ret), types))
    return out


def test_julia_ccalls_match_prototypes():
    protos = c_prototypes()
    calls = julia_ccalls()
    called = {c[0] for c in calls}
    # the binding covers the solver, the ensemble and the reverse mode
    assert {"mpm_create", "mpm_step", "mpm_download", "mpm_download_grid", "mpm_destroy", "mpm_step_energies",
            "mpm_batch_create", "mpm_batch_step", "mpm_batch_download", "mpm_batch_destroy",
            "mpm_fwd_checkpointed", "mpm_bwd", "mpm_abi_version", "mpm_last_error"} <= called
    for name, ret, types in calls:
        assert name in protos, name
        cret, ctypes_ = protos[name]
        # opaque handles (mpm_ctx*, mpm_batch*, instance arrays) may be passed as void pointers
        norm = lambda ts: [("void*" if t.startswith("mpm_instance_desc*") else t) for t in ts]
        assert ret == cret, (name, ret, cret)
        assert norm(types) == norm(ctypes_) or [t.replace("mpm_instance_desc*", "void*") for t in types] == \
            norm(ctypes_), (name, types, ctypes_)
