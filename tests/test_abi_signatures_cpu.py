"""Every function the ctypes binding declares has the header's return kind,
parameter count and, parameter by parameter, a ctypes type of the same kind
(pointer, float, double, int, 64-bit int, size_t): a float passed where the
library reads an int, or a missing argument, would go through ctypes
silently."""
import ctypes as C
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _prototypes(header=ROOT / "include" / "rtr.h"):
    txt = Path(header).read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w \t]*?[\s\*]+)\b([A-Za-z_]\w*)\s*\(([^;{}()]*(?:\([^()]*\)[^;{}()]*)*)\)\s*;",
                         txt):
        params = [p.strip() for p in m.group(3).split(",")]
        if params == ["void"] or params == [""]:
            params = []
        out[m.group(2)] = (m.group(1).split("\n")[-1].strip(), params)
    return out


def _kind_ret(r):
    r = r.replace("extern", "").strip()
    if r == "void":
        return None
    if r in ("rtr_status", "cudaError_t", "int"):
        return "i32"
    return _kind_c(r + " x")


def _kind_c(p):
    if "*" in p or "rtr_stream_t" in p:
        return "ptr"
    base = re.sub(r"\b(const|unsigned)\b", "", p).split()
    t = " ".join(base[:-1]) if len(base) > 1 else base[0]
    return {"float": "f32", "double": "f64", "int": "i32", "int32_t": "i32", "size_t": "size",
            "long long": "i64", "int64_t": "i64", "uint64_t": "u64", "uint32_t": "u32"}.get(t, t)


def _kind_py(t):
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return "ptr"
    for kind, cands in (("f32", (C.c_float,)), ("f64", (C.c_double,)), ("size", (C.c_size_t,)),
                        ("i64", (C.c_longlong, C.c_int64)), ("u64", (C.c_uint64, C.c_ulonglong)),
                        ("u32", (C.c_uint32, C.c_uint)), ("i32", (C.c_int, C.c_int32))):
        if t in cands:
            return kind
    return repr(t)


def _check(table, protos):
    checked = 0
    for name, (res, args) in table.items():
        if name not in protos:
            continue
        ret, params = protos[name]
        kr, kres = _kind_ret(ret), (None if res is None else _kind_py(res))
        assert kr == kres or {kr, kres} <= {"size", "u64"}, (name, ret, res)
        assert len(params) == len(args), (name, params, args)
        for p, a in zip(params, args):
            kc, kp = _kind_c(p), _kind_py(a)
            if {kc, kp} <= {"size", "u64"}:  # one unsigned 64-bit type on LP64 (ctypes aliases them)
                continue
            assert kc == kp, (name, p, a)
        checked += 1
    return checked


def test_binding_signatures_match_the_header(rtr):
    assert _check(rtr._SIG, _prototypes()) == len(rtr._SIG)  # every bound function is declared


def test_oracle_binding_signatures_match_its_header():
    import oracle as O
    assert _check(O._SIG, _prototypes(ROOT / "oracle" / "oracle.h")) == len(O._SIG)
