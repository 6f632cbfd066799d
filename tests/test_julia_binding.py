"""The Julia binding (vahana.jl_gb300/julia/VahanaGB300.jl) against the C ABI.

Julia is not available to run the binding, so this test reads it: every
`ccall((:vg_..., LIB), Ret, (ArgTypes...), ...)` must name a symbol the
library exports, pass as many arguments as include/vahana_gb300.h declares,
and use a Julia type compatible with each declared C type.  Calls through a
symbol held in a variable are checked against every symbol the enclosing
function (or its callers) can pass.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "vahana.jl_gb300", "julia", "VahanaGB300.jl")
HDR = os.path.join(ROOT, "include", "vahana_gb300.h")


def split_top(s):
    """Split at commas outside (), {} and []."""
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


def balanced(s, i):
    """s[i] is an opening parenthesis: the index after its match."""
    depth = 0
    for j in range(i, len(s)):
        if s[j] == "(":
            depth += 1
        elif s[j] == ")":
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError("unbalanced")


def header_decls():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    decls = {}
    for m in re.finditer(r"\b(vg_\w+)\s*\(", src):
        name = m.group(1)
        pre = src[max(0, m.start() - 40):m.start()]
        if "#define" in pre.splitlines()[-1] if pre.splitlines() else False:
            continue
        end = balanced(src, m.end() - 1)
        tail = src[end:end + 2].strip()
        if not tail.startswith(";"):
            continue
        args = split_top(src[m.end():end - 1])
        if args == ["void"]:
            args = []
        decls[name] = [re.sub(r"\s+", " ", a) for a in args]
    return decls


def ccalls(text):
    """(symbol or variable, arg types, offset) of every ccall."""
    out = []
    for m in re.finditer(r"ccall\(\(\s*(:?\w+)\s*,\s*LIB\s*\)\s*,", text):
        start = m.start() + len("ccall")
        end = balanced(text, start)
        parts = split_top(text[start + 1:end - 1])
        tup = parts[2]
        assert tup.startswith("(") and tup.endswith(")"), tup
        types = split_top(tup[1:-1])
        out.append((m.group(1), types, m.start()))
    return out


C_TO_JULIA = {
    "int": {"Cint", "Int32"}, "unsigned": {"Cuint", "UInt32"}, "uint32_t": {"UInt32", "Cuint"},
    "int32_t": {"Int32", "Cint"}, "uint64_t": {"UInt64", "Csize_t"}, "int64_t": {"Int64"},
    "double": {"Cdouble", "Float64"}, "float": {"Cfloat", "Float32"},
    "uint8_t": {"UInt8"}, "uint16_t": {"UInt16"},
}


def compatible(ctype, jtype):
    base = re.sub(r"\bconst\b", "", ctype).strip()
    base = re.sub(r"\s*\w+$", "", base) if not base.endswith("*") and " " in base else base
    if "*" in base:
        if "char" in base and "*" == base.replace(" ", "")[-1] and base.count("*") == 1:
            return jtype in ("Cstring", "Ptr{UInt8}", "Ptr{Cchar}", "Ptr{Cvoid}")
        return jtype.startswith("Ptr") or jtype.startswith("Ref") or jtype == "Cstring"
    base = base.replace("struct", "").strip()
    return jtype in C_TO_JULIA.get(base, {jtype})


def function_block(text, pos):
    """Text of the Julia function enclosing offset pos, and its name."""
    starts = [m for m in re.finditer(r"^function\s+(\w+)", text, flags=re.M) if m.start() < pos]
    if not starts:
        return "", ""
    m = starts[-1]
    nxt = re.search(r"^end\b", text[m.start():], flags=re.M)
    return text[m.start():m.start() + (nxt.end() if nxt else len(text))], m.group(1)


def test_binding_symbols_and_arities(vh):
    text = open(JL).read()
    decls = header_decls()
    exported = set(vh.exported_symbols())
    lib = vh.lib()
    calls = ccalls(text)
    assert len(calls) >= 40
    problems = []
    for sym, types, pos in calls:
        if sym.startswith(":"):
            cands = [sym[1:]]
        else:  # a symbol held in a variable: the function's literals, or its callers'
            block, fname = function_block(text, pos)
            cands = re.findall(r":(vg_\w+)", block)
            cands += re.findall(r"\b%s\(\s*\w+\s*,\s*:(vg_\w+)" % re.escape(fname), text)
            cands = sorted(set(cands))
            assert cands, "no candidate symbols for ccall((%s, LIB), ...)" % sym
        for name in cands:
            if name not in decls:
                problems.append("%s: not declared in the header" % name)
                continue
            if not hasattr(lib, name):
                problems.append("%s: not exported by the library" % name)
            if name not in exported:
                problems.append("%s: no ctypes signature" % name)
            if not sym.startswith(":"):
                continue  # arity of variable calls: checked below per function
            if len(types) != len(decls[name]):
                problems.append("%s: %d arguments, the header declares %d"
                                % (name, len(types), len(decls[name])))
                continue
            for k, (ct, jt) in enumerate(zip(decls[name], types)):
                if not compatible(ct, jt):
                    problems.append("%s argument %d: C %r vs Julia %r" % (name, k, ct, jt))
    # variable-symbol calls: every candidate's arity is one of the function's call arities
    for sym, types, pos in calls:
        if sym.startswith(":"):
            continue
        block, fname = function_block(text, pos)
        arities = {len(t) for s, t, p in calls if not s.startswith(":")
                   and function_block(text, p)[1] == fname}
        cands = set(re.findall(r":(vg_\w+)", block))
        cands |= set(re.findall(r"\b%s\(\s*\w+\s*,\s*:(vg_\w+)" % re.escape(fname), text))
        for name in cands:
            if name in decls and len(decls[name]) not in arities:
                problems.append("%s via %s(): header arity %d not among %s"
                                % (name, fname, len(decls[name]), sorted(arities)))
    assert problems == []


def test_every_symbol_literal_is_exported(vh):
    text = open(JL).read()
    lib = vh.lib()
    names = set(re.findall(r":(vg_\w+)", text))
    assert len(names) >= 30
    assert sorted(n for n in names if not hasattr(lib, n)) == []


@pytest.mark.parametrize("bad", ["int vg_x(int a, double b);"])
def test_header_parser_counts_arguments(bad):
    assert split_top("int a, double b, Ptr{Ptr{Cvoid}} c") == ["int a", "double b",
                                                              "Ptr{Ptr{Cvoid}} c"]
