"""The Julia glue (julia/gb300_glue.jl) against the C ABI it binds
(include/haplo_gb300.h), without Julia: every ccall names a declared entry
point, with the declared return type and one Julia type per C parameter that
passes the same machine type, and as many call arguments as types; every
mirrored struct has the C struct's fields, in order, with the same types.
CPU only."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "haplo_gb300.h")
GLUE = os.path.join(ROOT, "julia", "gb300_glue.jl")

JL_SCALAR = {"Cint": "int", "Int32": "int32_t", "Int64": "int64_t", "Float64": "double", "Float32": "float",
             "UInt64": "uint64_t", "UInt8": "uint8_t", "Cvoid": "void", "Cstring": "char*",
             "HxOpts": "hx_opts", "HxLoopOpts": "hx_loop_opts", "HxIterInfo": "hx_iter_info",
             "HxFitInfo": "hx_fit_info"}
OPAQUE = {"hx_ctx", "void"}          # a Ptr{Cvoid} may carry either


def _strip_comments(src):
    return re.sub(r"/\*.*?\*/", "", src, flags=re.S)


def c_type(decl):
    """'const double* q' -> 'double*'; 'uint64_t counts[16]' -> 'uint64_t*'."""
    decl = decl.strip()
    arr = decl.endswith("]")
    decl = re.sub(r"\[[^\]]*\]$", "", decl).strip()
    decl = decl.replace("const", " ")
    m = re.match(r"^\s*([A-Za-z_][A-Za-z0-9_]*)\s*([\s\*]*)\s*([A-Za-z_][A-Za-z0-9_]*)?\s*$", decl)
    assert m, decl
    base, stars = m.group(1), m.group(2).count("*")
    if arr:
        stars += 1
    if base == "char" and stars >= 1:
        return "char*" + "*" * (stars - 1)
    return base + "*" * stars


def header_functions():
    src = _strip_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"(?m)^\s*([A-Za-z_][A-Za-z0-9_ \*]*?)\s*\b(hx_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        ret, name, params = m.group(1), m.group(2), m.group(3)
        plist = [] if params.strip() in ("", "void") else [p for p in params.split(",")]
        out[name] = (c_type(ret + " r"), [c_type(p) for p in plist])
    return out


def header_structs():
    src = _strip_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"typedef struct (hx_[a-z_]+) \{(.*?)\}\s*\1\s*;", src, flags=re.S):
        fields = []
        for stmt in m.group(2).split(";"):
            stmt = stmt.strip()
            if not stmt:
                continue
            t, rest = stmt.split(None, 1)
            for name in rest.split(","):
                fields.append((name.strip(), t))
        out[m.group(1)] = fields
    return out


def jl_type(t):
    t = t.strip()
    m = re.match(r"^(Ptr|Ref)\{(.*)\}$", t)
    if m:
        return jl_type(m.group(2)) + "*"
    assert t in JL_SCALAR, "unmapped Julia type %s" % t
    return JL_SCALAR[t]


def _split_top(s):
    """Splits s at top-level commas (outside (), {}, [])."""
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur)
    return [p.strip() for p in parts]


def glue_ccalls():
    src = open(GLUE).read()
    src = re.sub(r"(?m)#.*$", "", src)
    calls = []
    for m in re.finditer(r"ccall\(", src):
        depth, a = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(src[a], 0)
            a += 1
        args = _split_top(src[m.end():a - 1])
        name = re.match(r"^\(:(hx_[a-z0-9_]+),\s*libhx\)$", args[0])
        assert name, args[0]
        types = args[2]
        assert types.startswith("(") and types.endswith(")"), types
        tlist = _split_top(types[1:-1])
        calls.append((name.group(1), args[1], tlist, args[3:]))
    return calls


def glue_structs():
    src = re.sub(r"(?m)#.*$", "", open(GLUE).read())
    out = {}
    for m in re.finditer(r"(?m)^struct (Hx[A-Za-z]+)\n(.*?)^end", src, flags=re.S):
        out[m.group(1)] = [tuple(x.strip() for x in ln.split("::")) for ln in m.group(2).strip().splitlines()]
    return out


def _same(cj, cc):
    if cj == cc:
        return True
    # Ptr{Cvoid} for an opaque handle, Ref{Ptr{Cvoid}} for hx_ctx**
    bj, bc = cj.rstrip("*"), cc.rstrip("*")
    return (len(cj) - len(bj)) == (len(cc) - len(bc)) and bj in OPAQUE and bc in OPAQUE


def test_glue_binds_only_declared_entry_points_with_matching_types():
    funcs = header_functions()
    calls = glue_ccalls()
    assert len(calls) >= 20
    for name, ret, tlist, cargs in calls:
        assert name in funcs, name
        cret, cparams = funcs[name]
        assert _same(jl_type(ret), cret), (name, ret, cret)
        assert len(tlist) == len(cparams), (name, tlist, cparams)
        for tj, tc in zip(tlist, cparams):
            assert _same(jl_type(tj), tc), (name, tj, tc)
        assert len(cargs) == len(tlist), (name, "arguments", cargs)


def test_glue_covers_the_reference_seams():
    called = {c[0] for c in glue_ccalls()}
    for must in ("hx_create", "hx_destroy", "hx_loglikelihood", "hx_em_accum", "hx_em_p_accum", "hx_update_q_accum",
                 "hx_update_p_accum", "hx_init_em", "hx_admixture_qn", "hx_fit", "hx_set_loop_opts",
                 "hx_qn_iteration", "hx_create_shared", "hx_fit_many"):
        assert must in called, must
    src = open(GLUE).read()
    for method in ("function _cu_admixture_base(", "function loglikelihood(d_cu::GB300Admix",
                   "function em!(d_cu::GB300Admix", "function em_p!(d_cu::GB300Admix",
                   "function update_q_cuda!(d_cu::GB300Admix", "function update_p_cuda!(d_cu::GB300Admix",
                   "function init_em!(d::AdmixData2, g, iter::Integer, d_cu::GB300Admix",
                   "function admixture_qn!(d::AdmixData2, g, n_iter::Integer, rtol, d_cu::GB300Admix"):
        assert method in src, method


@pytest.mark.parametrize("jl,c", [("HxOpts", "hx_opts"), ("HxLoopOpts", "hx_loop_opts"),
                                  ("HxIterInfo", "hx_iter_info"), ("HxFitInfo", "hx_fit_info")])
def test_glue_structs_mirror_the_header(jl, c):
    js, cs = glue_structs()[jl], header_structs()[c]
    assert [n for n, _ in js] == [n for n, _ in cs]
    for (_, tj), (_, tc) in zip(js, cs):
        assert jl_type(tj) == tc, (jl, tj, tc)


def test_parser_sees_every_header_function():
    # guards the header parser itself: it finds as many functions as the ABI test's regex
    src = _strip_comments(open(HEADER).read())
    names = set(re.findall(r"\b(hx_[a-z0-9_]+)\s*\(", src))
    assert names == set(header_functions())
