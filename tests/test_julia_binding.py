"""The Julia binding (the julia/ package: src/PTDiffusion.jl and its ChainRulesCore
extension) against the C ABI it calls.

There is no Julia toolchain here, so the binding is checked as text: its
`PtdParams` mirror must list the members of `ptd_params` (include/ptd.h) in
order with matching types (Julia lays out an isbits struct with C's rules,
so equal member lists mean equal layouts), every `ccall` must name an entry
point the header declares with the same return type, argument count and
compatible argument types, and its enum tables must carry the header's
values."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JLPKG = os.path.join(ROOT, "pseudotransientdiffusion.jl_gb300", "julia")
JL = os.path.join(JLPKG, "src", "PTDiffusion.jl")
JLEXT = os.path.join(JLPKG, "ext", "PTDiffusionChainRulesCoreExt.jl")
HEADER = os.path.join(ROOT, "include", "ptd.h")

C_SCALAR = {"int32_t": "Int32", "int": "Int32", "double": "Float64", "float": "Float32", "int64_t": "Int64"}
OPAQUE = {"ptd_ctx", "ptd_adj", "ptd_batch", "void"}


def _header():
    with open(HEADER) as fh:
        text = fh.read()
    return re.sub(r"/\*.*?\*/", " ", text, flags=re.S)


def _julia():
    with open(JL) as fh:
        return fh.read()


def _split_top(s):
    """Split s at commas outside (), {} and []."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _matching(s, i):
    """Index of the bracket closing the one at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        if s[j] in "({[":
            depth += 1
        elif s[j] in ")}]":
            depth -= 1
            if depth == 0:
                return j
    raise ValueError("unbalanced")


def c_struct_members(text, name):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    members = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        for n in names.split(","):
            n = n.strip()
            m = re.match(r"(\w+)\[(\d+)\]$", n)
            if m:
                members.append((m.group(1), "NTuple{%s,%s}" % (m.group(2), C_SCALAR[ctype])))
            else:
                members.append((n, C_SCALAR[ctype]))
    return members


def julia_struct_fields(text, name):
    body = re.search(r"mutable struct %s\n(.*?)\nend" % name, text, re.S).group(1)
    fields = []
    for line in body.splitlines():
        line = line.split("#")[0]
        for item in line.split(";"):
            item = item.strip()
            if item:
                n, t = item.split("::")
                fields.append((n.strip(), t.strip()))
    return fields


def c_prototypes(text):
    protos = {}
    for m in re.finditer(r"PTD_API\s+([\w\s\*]+?)\s*\b(ptd_\w+)\s*\((.*?)\)\s*;", text, re.S):
        ret, name, params = " ".join(m.group(1).split()), m.group(2), " ".join(m.group(3).split())
        args = [] if params in ("", "void") else [_c_param(p) for p in params.split(",")]
        protos[name] = (ret, args)
    return protos


def _c_param(p):
    """(base type, pointer depth) of one C parameter."""
    p = p.replace("const", " ")
    depth = p.count("*") + p.count("[")
    toks = re.findall(r"\w+", re.sub(r"\[\d*\]", "", p))
    base = {"int": "int32_t"}.get(toks[0], toks[0])   # C int and Julia's Cint are 32-bit here
    return ("opaque" if base in OPAQUE else base, depth)


def _julia_arg(t):
    """(base type, pointer depth) of one ccall argument type."""
    m = re.match(r"(Ptr|Ref)\{(.*)\}$", t)
    if m:
        base, depth = _julia_arg(m.group(2))
        return base, depth + 1
    return {"Cvoid": "opaque", "Int32": "int32_t", "Cint": "int32_t", "Float64": "double",
            "Cdouble": "double", "PtdParams": "ptd_params", "Int64": "int64_t"}[t], 0


def julia_ccalls(text):
    calls = []
    for m in re.finditer(r"ccall\(", text):
        i = m.end() - 1
        items = _split_top(text[i + 1:_matching(text, i)])
        sym = re.match(r"\(:(\w+),\s*libptd\)", items[0]).group(1)
        argt = items[2].strip()
        assert argt.startswith("(") and argt.endswith(")"), argt
        calls.append((sym, items[1].strip(), [a for a in _split_top(argt[1:-1]) if a]))
    return calls


def test_params_mirror_matches_the_header():
    c = c_struct_members(_header(), "ptd_params")
    jl = julia_struct_fields(_julia(), "PtdParams")
    assert jl == c


def test_every_ccall_matches_its_prototype():
    protos = c_prototypes(_header())
    calls = julia_ccalls(_julia())
    assert len(calls) >= 10
    ret_map = {"Cint": "int", "Cvoid": "void", "Cstring": "const char*"}
    for sym, ret, args in calls:
        assert sym in protos, sym
        cret, cargs = protos[sym]
        assert ret_map[ret] == cret.replace(" *", "*"), (sym, ret, cret)
        assert len(args) == len(cargs), (sym, args, cargs)
        for a, (cbase, cdepth) in zip(args, cargs):
            base, depth = _julia_arg(a)
            assert (base, depth) == (cbase, cdepth), (sym, a, cbase, cdepth)


def test_enum_tables_match_the_header():
    h = _header()
    jl = _julia()
    enum = dict((k, int(v)) for k, v in re.findall(r"\b(PTD_\w+)\s*=\s*(\d+)", h))
    models = dict((k, int(v)) for k, v in re.findall(r":(\w+) => Int32\((\d+)\)",
                                                    re.search(r"const MODEL = Dict\((.*?)\)\n", jl).group(1)))
    precs = dict((k, int(v)) for k, v in re.findall(r":(\w+) => Int32\((\d+)\)",
                                                   re.search(r"const PRECISION = Dict\((.*?)\)\n", jl, re.S).group(1)))
    assert models and precs
    for k, v in models.items():
        assert enum["PTD_MODEL_" + k.upper()] == v, k
    for k, v in precs.items():
        assert enum["PTD_PREC_" + k.upper()] == v, k
    assert int(re.search(r"const PTD_OK = Cint\((\d+)\)", jl).group(1)) == enum["PTD_OK"]


def test_rrule_is_a_package_extension():
    """The rrule lives in a package extension declared in Project.toml, so it
    does not depend on the order in which ChainRulesCore and PTDiffusion load."""
    with open(os.path.join(JLPKG, "Project.toml")) as fh:
        proj = fh.read()
    assert re.search(r'^name = "PTDiffusion"$', proj, re.M)
    assert re.search(r'^\[weakdeps\]\nChainRulesCore = "d360d2e6-b24c-11e9-a2a3-2a2ae2dbcce4"$', proj, re.M)
    assert re.search(r'^\[extensions\]\nPTDiffusionChainRulesCoreExt = "ChainRulesCore"$', proj, re.M)
    with open(JLEXT) as fh:
        ext = fh.read()
    assert "module PTDiffusionChainRulesCoreExt" in ext
    assert "function ChainRulesCore.rrule(::typeof(misfit), a::AdjointSolver, m, H0, Ht)" in ext
    assert "isdefined(Main" not in _julia()
    assert "forward!" in _julia() and "gradient!" in _julia()
