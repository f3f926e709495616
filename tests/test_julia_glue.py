"""The Julia glue (volumefluxes.jl_gb300/julia/VolumeFluxesSM103.jl) against the C
header: every `ccall((:sym, LIB), Ret, (Args...), ...)` names a symbol that
include/volumefluxes_sm103.h declares, passes as many arguments as the C
prototype takes, and uses Julia types that match the C types (scalars by
width, pointers by pointee). No Julia toolchain exists here, so the file is
checked as text; the VfConfig mirror is checked field by field against the
vf_config struct."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
GLUE = ROOT / "volumefluxes.jl_gb300" / "julia" / "VolumeFluxesSM103.jl"
HEADER = ROOT / "include" / "volumefluxes_sm103.h"


def _strip_c_comments(s: str) -> str:
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


def c_prototypes() -> dict:
    """{name: (return type, [parameter types])} of every vf_* function."""
    text = _strip_c_comments(HEADER.read_text())
    text = re.sub(r"^\s*#.*$", " ", text, flags=re.M)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(vf_\w+)\s*\(([^;{}]*?)\)\s*;", text):
        ret, name, params = " ".join(m.group(1).split()), m.group(2), " ".join(m.group(3).split())
        if ret.startswith("typedef"):
            continue
        types = []
        if params not in ("", "void"):
            for p in params.split(","):
                p = p.strip()
                # drop the parameter name (last identifier not part of the type)
                t = re.sub(r"\b[A-Za-z_]\w*\s*$", "", p).strip()
                types.append(" ".join(t.replace("*", " * ").split()))
        out[name] = (" ".join(ret.replace("*", " * ").split()), types)
    return out


def _split_top(s: str) -> list:
    """Split at commas outside (), {} and []."""
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur).strip())
    return parts


def julia_ccalls() -> list:
    """(symbol, return type, [argument types], [argument values], line) of every ccall."""
    text = GLUE.read_text()
    text = re.sub(r"#[^\n]*", "", text)  # comments
    calls = []
    for m in re.finditer(r"ccall\(", text):
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(text[i], 0)
            i += 1
        body = text[m.end():i - 1]
        args = _split_top(body)
        sym = re.match(r"\(\s*:(\w+)\s*,\s*LIB\s*\)", args[0])
        assert sym, args[0]
        tup = args[2].strip()
        assert tup.startswith("(") and tup.endswith(")"), tup
        types = _split_top(tup[1:-1])
        line = text[:m.start()].count("\n") + 1
        calls.append((sym.group(1), args[1].strip(), types, args[3:], line))
    return calls


SCALARS = {"Float64": {"double"}, "Float32": {"float"}, "Int32": {"int32_t", "int"}, "Cint": {"int", "int32_t"},
           "Int64": {"int64_t"}, "Cvoid": {"void"}, "Cstring": {"const char *"}}


def _pointee(c: str) -> str:
    """'const double *' -> 'double'; 'vf_handle * const *' -> 'vf_handle *'."""
    c = c.strip()
    assert c.endswith("*"), c
    inner = c[:-1].strip()
    if inner.endswith("const"):
        inner = inner[:-5].strip()
    return inner[6:].strip() if inner.startswith("const ") else inner


def compatible(jt: str, ct: str) -> bool:
    jt = jt.replace(" ", "")
    if jt in SCALARS:
        return ct in SCALARS[jt]
    m = re.fullmatch(r"(Ptr|Ref)\{(.+)\}", jt)
    if not m or not ct.endswith("*"):
        return False
    inner, pointee = m.group(2), _pointee(ct)
    if inner == "Cvoid":
        return True  # an untyped pointer: any C pointer (handles, NULL options, raw buffers)
    if pointee == "void":
        return inner in ("T", "Cvoid", "Float64", "Float32")  # a raw buffer of the state's real type
    if inner == "VfConfig":
        return pointee == "vf_config"
    if inner.startswith("Ptr{"):
        return pointee.endswith("*")  # a pointer to handles / out-handles
    return pointee in SCALARS.get(inner, set())


def test_glue_file_exists_and_has_ccalls():
    calls = julia_ccalls()
    assert len(calls) >= 25
    # the entry points a scenario script needs
    syms = {c[0] for c in calls}
    for s in ("vf_create", "vf_destroy", "vf_step", "vf_simulate", "vf_set_interior_state", "vf_download_state",
              "vf_upload_bottom", "vf_last_error", "vf_adjoint_forward", "vf_adjoint_backward", "vf_server_submit"):
        assert s in syms, s


@pytest.mark.parametrize("call", julia_ccalls(), ids=lambda c: f"{c[0]}@{c[4]}")
def test_ccall_matches_the_header(call):
    sym, ret, types, values, line = call
    protos = c_prototypes()
    assert sym in protos, f"{sym} (line {line}) is not declared in the header"
    cret, ctypes = protos[sym]
    assert len(types) == len(ctypes), f"{sym} line {line}: {len(types)} argument types, C takes {len(ctypes)}"
    assert len(values) == len(types), f"{sym} line {line}: {len(values)} values for {len(types)} types"
    assert compatible(ret, cret), f"{sym} line {line}: returns {ret}, C returns {cret}"
    for k, (jt, ct) in enumerate(zip(types, ctypes)):
        assert compatible(jt, ct), f"{sym} line {line}: argument {k + 1} is {jt}, C has {ct}"


def test_every_adjoint_and_server_call_checks_its_return_code():
    """Calls returning a status are wrapped in check/adjoint_check/server_check,
    except the destructors (which have nothing to report)."""
    text = re.sub(r"#[^\n]*", "", GLUE.read_text())
    for m in re.finditer(r"ccall\(\(:(vf_\w+)", text):
        sym = m.group(1)
        if sym.endswith(("_destroy", "_last_error")):
            continue
        before = text[max(0, m.start() - 40):m.start()]
        assert re.search(r"(check|adjoint_check|server_check)\([^()]*$", before) or \
            re.search(r"rc = $", before), f"{sym}: return code not checked"


def test_vfconfig_mirror_matches_the_header_struct():
    text = re.sub(r"#[^\n]*", "", GLUE.read_text())
    body = re.search(r"struct VfConfig\n(.*?)\nend", text, flags=re.S).group(1)
    jfields = [f.split("::") for f in re.split(r"[;\n]", body) if "::" in f]
    jfields = [(a.strip(), b.strip()) for a, b in jfields]
    raw = HEADER.read_text()
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define (\w+) (\d+)\b", raw)}
    h = _strip_c_comments(raw)
    cbody = re.search(r"typedef struct vf_config\s*\{(.*?)\}\s*vf_config\s*;", h, flags=re.S).group(1)
    cfields = []
    for decl in cbody.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        ctype, rest = decl.split(" ", 1)
        for d in rest.split(","):
            m = re.fullmatch(r"(\w+)((?:\[\w+\])*)", d.strip())
            assert m, decl
            n = 1
            for dim in re.findall(r"\[(\w+)\]", m.group(2)):
                n *= int(dim) if dim.isdigit() else consts[dim]
            cfields.append((m.group(1), ctype, n))
    assert [f[0] for f in jfields] == [f[0] for f in cfields]
    scalar = {"int32_t": "Int32", "double": "Float64", "int": "Int32"}
    for (jn, jt), (cn, ct, n) in zip(jfields, cfields):
        want = scalar[ct] if n == 1 else f"NTuple{{{n},{scalar[ct]}}}"
        assert jt.replace(" ", "") == want, (jn, jt, want)
