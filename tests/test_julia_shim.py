"""The Julia ccall shim against the C header, without Julia.

Julia is not installed here, so the shim (trixiparticles.jl_gb300/julia/TrixiParticlesGB300.jl)
cannot run.  What can be checked on text: its TpConfig mirrors `tp_config` field by field with
the same C types, every `ccall` names an exported function with the header's argument list, the
dispatch selects `Semidiscretization{<:GB300Backend}` through the reference's first type
parameter (src/general/semidiscretization.jl:78), the search is looked up through the
reference's handler accessor (src/general/neighborhood_search.jl:397-416), and the Julia block
of the repository's integration guide makes the same calls.
"""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "tp_wcsph.h"
SHIM = ROOT / "trixiparticles.jl_gb300" / "julia" / "TrixiParticlesGB300.jl"
INTEGRATION = ROOT / "INTEGRATION.md"


def _strip_c_comments(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def _split_top(s):
    """Split at commas outside (), {}, [] and string literals."""
    out, depth, cur, quote = [], 0, [], None
    for ch in s:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        elif ch == "," and depth == 0:
            out.append("".join(cur).strip())
            cur = []
            continue
        cur.append(ch)
    if "".join(cur).strip():
        out.append("".join(cur).strip())
    return out


def _balanced(text, start):
    """Text between the parenthesis at `start` and its partner."""
    depth = 0
    for k in range(start, len(text)):
        if text[k] == "(":
            depth += 1
        elif text[k] == ")":
            depth -= 1
            if depth == 0:
                return text[start + 1:k]
    raise ValueError("unbalanced")


# ---- header side -------------------------------------------------------------------------
def _c_kind(ctype):
    t = ctype.replace("const", "").replace(" ", "")
    t = re.sub(r"\[\d*\]$", "*", t)
    kinds = {
        "tp_handle*": "ptr", "tp_batch*": "ptr", "void*": "ptr",
        "tp_handle**": "ptrptr", "tp_batch**": "ptrptr",
        "tp_handle**const": "ptrarray", "tp_handle*const*": "ptrarray",
        "tp_config*": "cfg*", "double*": "f64*", "int32_t*": "i32*", "int*": "i32*",
        "double": "f64", "int64_t": "i64", "int32_t": "i32", "int": "i32",
        "tp_status": "i32", "char*": "str",
    }
    return kinds.get(t, t)


def header_prototypes():
    text = _strip_c_comments(HEADER.read_text())
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w \*]*?)\b(tp_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text):
        ret, name, params = m.group(1), m.group(2), m.group(3)
        kinds = []
        for p in _split_top(params):
            if p in ("", "void"):
                continue
            pm = re.match(r"(.*?)([A-Za-z_]\w*)\s*(\[\d*\])?$", p.strip())
            ptype = pm.group(1) + (pm.group(3) or "")
            if "*const*" in ptype.replace(" ", ""):
                kinds.append("ptrarray")
            else:
                kinds.append(_c_kind(ptype))
        protos[name] = (_c_kind(ret.strip()), kinds)
    return protos


def header_config_fields():
    text = _strip_c_comments(HEADER.read_text())
    body = re.search(r"typedef struct tp_config\s*\{(.*?)\}\s*tp_config\s*;", text, re.S).group(1)
    fields = []
    for line in body.split(";"):
        line = line.strip()
        if not line:
            continue
        m = re.match(r"(.*?)([A-Za-z_]\w*)\s*(\[(\d+)\])?$", line)
        ctype, name, arr = m.group(1).strip(), m.group(2), m.group(4)
        fields.append((name, ctype, int(arr) if arr else None))
    return fields


# ---- Julia side --------------------------------------------------------------------------
JULIA_KIND = {
    "Ptr{Cvoid}": "ptr", "Ref{Ptr{Cvoid}}": "ptrptr", "Ptr{Ptr{Cvoid}}": "ptrarray",
    "Ref{TpConfig}": "cfg*", "CuPtr{Float64}": "f64*", "Ptr{Float64}": "f64*",
    "CuPtr{Int32}": "i32*", "Ptr{Int32}": "i32*", "Float64": "f64", "Int64": "i64",
    "Int32": "i32", "Cint": "i32", "Cstring": "str",
}
JULIA_FIELD = {"Int32": ("int32_t", None), "Int64": ("int64_t", None),
               "Float64": ("double", None), "NTuple{3, Float64}": ("double", 3)}


def julia_ccalls(text):
    calls = []
    for m in re.finditer(r"ccall\(", text):
        inner = _balanced(text, m.end() - 1)
        parts = _split_top(inner)
        target = re.match(r"\(:(tp_[a-z0-9_]+),\s*libtp\)", parts[0])
        assert target, parts[0]
        ret = parts[1]
        types = parts[2].strip()
        assert types.startswith("(") and types.endswith(")"), types
        tlist = _split_top(types[1:-1])
        calls.append((target.group(1), ret, tlist, parts[3:]))
    return calls


def julia_config_fields(text):
    body = re.search(r"struct TpConfig\n(.*?)\nend", text, re.S).group(1)
    fields = []
    for item in re.split(r"[;\n]", body):
        item = item.strip()
        if item:
            name, jtype = item.split("::")
            fields.append((name.strip(), jtype.strip()))
    return fields


def _integration_julia_block():
    text = INTEGRATION.read_text()
    blocks = re.findall(r"```julia\n(.*?)```", text, re.S)
    assert blocks, "the integration guide has no Julia block"
    return "\n".join(blocks)


# ---- tests -------------------------------------------------------------------------------
@pytest.mark.parametrize("source", ["shim", "integration"])
def test_tpconfig_mirrors_header(source):
    text = SHIM.read_text() if source == "shim" else _integration_julia_block()
    jl = julia_config_fields(text)
    c = header_config_fields()
    assert [n for n, _ in jl] == [n for n, _, _ in c]
    for (name, jtype), (_, ctype, arr) in zip(jl, c):
        assert JULIA_FIELD[jtype] == (ctype, arr), name


@pytest.mark.parametrize("source", ["shim", "integration"])
def test_ccalls_match_header_prototypes(source):
    text = SHIM.read_text() if source == "shim" else _integration_julia_block()
    protos = header_prototypes()
    calls = julia_ccalls(text)
    assert calls
    for name, ret, tlist, args in calls:
        assert name in protos, f"{name} is not declared in tp_wcsph.h"
        c_ret, c_args = protos[name]
        assert JULIA_KIND[ret] == c_ret, (name, ret, c_ret)
        assert [JULIA_KIND[t] for t in tlist] == c_args, (name, tlist, c_args)
        assert len(args) == len(tlist), (name, args)


def test_shim_covers_the_hot_path_calls():
    names = {c[0] for c in julia_ccalls(SHIM.read_text())}
    for n in ("tp_create", "tp_set_stream", "tp_set_wall", "tp_set_fluid_mass", "tp_kick",
              "tp_drift", "tp_sync", "tp_destroy", "tp_last_error", "tp_integrate_ck2n54",
              "tp_adjoint_forward", "tp_adjoint_backward"):
        assert n in names, n


def test_dispatch_uses_the_backend_type_parameter_and_handler():
    text = SHIM.read_text()
    # BACKEND is the first type parameter of the reference's Semidiscretization
    assert re.search(r"const GB300Semi = Semidiscretization\{<:GB300Backend\}", text)
    assert "NamedTuple{(:semi, :split_integration_data), <:Tuple{GB300Semi, Any}}" in text
    for fn in ("kick!", "drift!"):
        assert re.search(rf"function TrixiParticles\.{fn}\([^)]*p::GB300Params", text), fn
    # the search comes from semi.neighborhood_search_handler via the reference's accessor
    assert "TrixiParticles.get_neighborhood_search(fluid, fluid, semi)" in text
    assert "neighborhood_searches" not in text
    # an immutable Semidiscretization cannot carry a finalizer: the handle is keyed elsewhere
    assert "finalizer(" in text and "WeakKeyDict" in text
    assert "finalizer(_ -> " not in text


def test_integration_shows_the_shim_binding():
    block = _integration_julia_block()
    assert "invoke(" not in block
    assert "Semidiscretization{<:GB300Backend}" in block
    shim = SHIM.read_text()
    for name, ret, tlist, _ in julia_ccalls(block):
        shim_sig = {(n, r, tuple(t)) for n, r, t, _ in julia_ccalls(shim)}
        assert (name, ret, tuple(tlist)) in shim_sig, name
