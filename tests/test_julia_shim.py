"""The Julia binding (julia/*.jl) against the C header, on the CPU.

Julia is not installed here, so the shim cannot run; this test reads it as
text and checks what a mismatch would break silently at run time:
  - every `ccall((:name, libkvmc), Cint, (argtypes...), ...)` names a
    function declared in include/kvmc.h, with as many arguments as the
    prototype and a Julia type of the same width and kind for each;
  - every struct the shim passes by reference (ModelDesc, BatchDesc,
    SweepStats, LatticeDesc, Link) has the C struct's fields in the same
    order with the same types;
  - the Carlo callbacks of the reference's plugin surface are defined, and
    `sweep!` runs the fused n-proposal call (kvmc_sweep with
    proposals_per_sweep), not one library call per proposal by default.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kvmc.h")
JULIA = [os.path.join(ROOT, "julia", f) for f in ("KagomeVMC.jl", "KagomeVMCChainRules.jl")]

STRUCTS = {"kvmc_lattice_desc": "LatticeDesc", "kvmc_link": "Link", "kvmc_model_desc": "ModelDesc",
           "kvmc_batch_desc": "BatchDesc", "kvmc_sweep_stats": "SweepStats"}
SCALAR = {"int32_t": {"Int32", "Cint"}, "int64_t": {"Int64"}, "uint64_t": {"UInt64"}, "double": {"Float64", "Cdouble"},
          "size_t": {"Csize_t", "UInt64"}}
POINTEE = {"int32_t": {"Int32", "Cint"}, "int64_t": {"Int64"}, "double": {"Float64"}, "float": {"Float32"},
           "char": {"UInt8", "Cchar"}, "void": {"Cvoid"}, "kvmc_handle": {"Cvoid"}, "kvmc_link": {"Link"}}


def _strip_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def header_prototypes():
    src = _strip_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"KVMC_API\s+int\s+(\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.S):
        args = [a.strip() for a in m.group(2).replace("\n", " ").split(",") if a.strip()]
        out[m.group(1)] = [a for a in args if a != "void"]
    return out


def c_arg_type(decl):
    """'const int32_t *bonds' -> ('int32_t', 1); 'kvmc_handle **out' -> ('kvmc_handle', 2)."""
    d = decl.replace("const", " ")
    stars = d.count("*")
    words = d.replace("*", " ").split()
    return words[0], stars


def julia_ok(ctype, stars, jt):
    jt = jt.strip()
    if stars == 0:
        return jt in SCALAR[ctype]
    m = re.fullmatch(r"(Ptr|Ref)\{(.+)\}", jt)
    if not m:
        return False
    inner = m.group(2)
    if stars == 2:
        return m.group(1) == "Ref" and inner == "Ptr{Cvoid}"
    if ctype in STRUCTS:
        return inner == STRUCTS[ctype] and (m.group(1) == "Ref" or ctype == "kvmc_link")
    return inner in POINTEE[ctype]


def split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur)
    return [p.strip() for p in parts if p.strip()]


def julia_ccalls():
    out = []
    for f in JULIA:
        src = open(f).read()
        for m in re.finditer(r"ccall\(\(:(\w+),\s*libkvmc\),\s*Cint,\s*\(([^()]*)\)", src):
            out.append((os.path.basename(f), m.group(1), split_top(m.group(2))))
    return out


def test_every_ccall_matches_its_prototype():
    protos = header_prototypes()
    calls = julia_ccalls()
    assert len(calls) >= 20
    for fname, name, jargs in calls:
        assert name in protos, f"{fname}: {name} is not declared in include/kvmc.h"
        cargs = protos[name]
        assert len(jargs) == len(cargs), (fname, name, jargs, cargs)
        for ca, ja in zip(cargs, jargs):
            ctype, stars = c_arg_type(ca)
            assert julia_ok(ctype, stars, ja), f"{fname}: {name}: C '{ca}' passed as Julia '{ja}'"


def c_struct_fields(name):
    src = _strip_comments(open(HEADER).read())
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r"\s*;", src)
    fields = []
    for line in m.group(1).split(";"):
        line = line.replace("const", " ").strip()
        if not line:
            continue
        ptr = "*" in line
        words = line.replace("*", " ").replace(",", " ").split()
        ctype, names = words[0], words[1:]
        for n in names:
            arr = re.fullmatch(r"(\w+)\[(\d+)\]", n)
            fields.append((arr.group(1) if arr else n, ctype, ptr, int(arr.group(2)) if arr else 0))
    return fields


def julia_struct_fields(name):
    src = open(JULIA[0]).read()
    m = re.search(r"struct " + name + r"\n(.*?)\nend", src, flags=re.S)
    return [tuple(x.strip() for x in line.split("::")) for line in m.group(1).strip().split("\n")]


def test_structs_match_the_header():
    for cname, jname in STRUCTS.items():
        cf, jf = c_struct_fields(cname), julia_struct_fields(jname)
        assert [f[0] for f in cf] == [f[0] for f in jf], (cname, cf, jf)
        for (fn, ctype, ptr, arr), (_, jt) in zip(cf, jf):
            if ptr:
                assert re.fullmatch(r"Ptr\{(\w+)\}", jt) and jt[4:-1] in POINTEE[ctype], (cname, fn, jt)
            elif arr:
                assert jt == f"NTuple{{{arr},{next(iter(sorted(SCALAR[ctype])))}}}" or \
                    any(jt == f"NTuple{{{arr},{t}}}" for t in SCALAR[ctype]), (cname, fn, jt)
            else:
                assert jt in SCALAR[ctype], (cname, fn, jt)


def test_carlo_callbacks_and_fused_sweep():
    src = open(JULIA[0]).read()
    for cb in ("Carlo.init!", "Carlo.sweep!", "Carlo.measure!", "Carlo.register_evaluables",
               "Carlo.write_checkpoint", "Carlo.read_checkpoint!"):
        assert f"function {cb}(" in src, cb
    body = src[src.index("function Carlo.sweep!("):]
    body = body[:body.index("\nend")]
    assert "kvmc_sweep(mc.h, mc.proposals_per_sweep)" in body
    # the default cadence is min(N_up, N_down) proposals per sweep! call
    assert 'get(params, :proposals_per_sweep, nocc)' in src and "nocc = min(params[:N_up], params[:N_down])" in src


def test_constants_match_the_header():
    """Every KVMC_* constant the Julia module defines has the header's value."""
    hdr = open(os.path.join(ROOT, "include", "kvmc.h")).read()
    consts = re.findall(r"const (KVMC_\w+) = Int32\((-?\d+)\)", open(JULIA[0]).read())
    assert len(consts) >= 10
    for name, val in consts:
        m = re.search(r"\b" + name + r"\s*=\s*(-?\d+)", hdr) or re.search(r"#define\s+" + name + r"\s+(-?\d+)", hdr)
        assert m and int(m.group(1)) == int(val), (name, val)
