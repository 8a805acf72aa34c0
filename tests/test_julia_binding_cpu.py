"""Static check of the Julia drop-in module (no Julia on either machine, so it cannot
run): every ccall names a function that include/gpugraphs.h declares and passes it as
many arguments as the declaration has parameters."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpugraphs.h")
JULIA = os.path.join(ROOT, "gpugraphs.jl_gb300", "julia", "GPUGraphs", "src", "GPUGraphs.jl")


def _split_top(s):
    """Split s at commas that are not nested in brackets."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [x.strip() for x in out if x.strip()]


def header_arity():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"^(?:int|int64_t|const char\*)\s+(gg_\w+)\s*\(([^;]*?)\)\s*;", src, re.M | re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(_split_top(params))
    return out


def julia_ccalls():
    src = open(JULIA).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(gg_\w+),\s*LIB\),\s*\w+,\s*\(", src):
        # the argument-type tuple starts at the '(' matched last; find its closing bracket
        i = m.end() - 1
        depth = 0
        for j in range(i, len(src)):
            if src[j] == "(":
                depth += 1
            elif src[j] == ")":
                depth -= 1
                if depth == 0:
                    break
        types = _split_top(src[i + 1:j])
        # the call arguments follow the type tuple up to the ccall's closing bracket
        k, depth = j + 1, 1
        start = k
        while depth > 0:
            if src[k] in "([{":
                depth += 1
            elif src[k] in ")]}":
                depth -= 1
            k += 1
        args = _split_top(src[start:k - 1].lstrip(","))
        calls.append((m.group(1), len(types), len(args)))
    return calls


def test_every_ccall_matches_the_header():
    decl = header_arity()
    calls = julia_ccalls()
    assert len(calls) >= 20
    for name, ntypes, nargs in calls:
        assert name in decl, name
        assert ntypes == decl[name], (name, ntypes, decl[name])
        assert nargs == ntypes, (name, nargs, ntypes)


def julia_exports():
    src = open(JULIA).read()
    m = re.search(r"^export\s+(.*?)(?:\n\s*\n|\n#)", src, re.M | re.S)
    assert m, "no export statement"
    return {x.strip() for x in m.group(1).replace("\n", " ").split(",") if x.strip()}


def test_module_exports_every_reference_name():
    """The drop-in module exports every name the reference's module exports
    (tests/golden/reference_exports.json, transcribed from src/GPUGraphs.jl:25-51),
    and defines each exported type."""
    import json
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_exports.json")))
    exported = julia_exports()
    missing = [n for n in ref["exports"] if n not in exported]
    assert not missing, missing
    src = open(JULIA).read()
    for name in ref["exports"]:
        if name[0].isupper() and not name.startswith("GPUGraphs_"):
            assert re.search(r"(struct|abstract type)\s+%s\b" % re.escape(name), src), name
