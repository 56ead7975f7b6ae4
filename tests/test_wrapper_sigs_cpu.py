"""The ctypes signatures of the Python wrapper against the C prototypes in
the public headers (include/*.h): same argument count, and per argument the same kind
(integer / floating / pointer) and size, so no call passes an int where the
header takes an int64_t or a float where it takes a double."""
import ctypes
import os
import re

import pytest

import gbblas

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_INT = {"int": 4, "int32_t": 4, "int64_t": 8, "uint64_t": 8, "uint32_t": 4, "size_t": 8, "char": 1,
        "unsigned long": 8, "long": 8, "unsigned": 4, "gb_status": 4}
_FLT = {"float": 4, "double": 8}


def _c_kind(decl):
    """('ptr',) / ('int', size) / ('float', size) / None (void) of a C parameter or return type."""
    t = re.sub(r"\b(const|struct|enum)\b", " ", decl)
    if "*" in t or "[" in t:
        return ("ptr",)
    words = t.split()
    if not words or words == ["void"]:
        return None
    # drop the parameter name when present (the last word after a type)
    for n in (2, 1):
        base = " ".join(words[:n])
        if base in _INT:
            return ("int", _INT[base])
        if base in _FLT:
            return ("float", _FLT[base])
    if words[0].startswith("gb_"):   # the library's enums
        return ("int", 4)
    raise ValueError("unknown C type: %r" % decl)


def _py_kind(t):
    if t is None:
        return None
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return ("ptr",)
    if t in (ctypes.c_float, ctypes.c_double):
        return ("float", ctypes.sizeof(t))
    return ("int", ctypes.sizeof(t))


def _prototypes():
    import glob
    text = "\n".join(open(f).read() for f in sorted(glob.glob(os.path.join(REPO, "include", "*.h"))))
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    text = re.sub(r"^\s*#[^\n]*", " ", text, flags=re.M)   # preprocessor lines
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(gb_\w+)\s*\(([^;{}()]*)\)\s*;", text):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith("typedef"):
            continue
        params = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        protos[name] = (ret, params)
    return protos


PROTOS = _prototypes()


def test_the_header_parses():
    assert len(PROTOS) > 40 and "gb_sgemm" in PROTOS and "gb_workspace_query" in PROTOS


@pytest.mark.parametrize("name", sorted(gbblas._SIGS))
def test_wrapper_signature_matches_header(name):
    assert name in PROTOS, "wrapper declares %s, the header does not" % name
    ret, params = PROTOS[name]
    args, res = gbblas._SIGS[name]
    assert len(args) == len(params), (name, params)
    for i, (p, a) in enumerate(zip(params, args)):
        assert _c_kind(p) == _py_kind(a), (name, i, p, a)
    assert _c_kind(ret) == _py_kind(res), (name, ret, res)


STRUCTS = {"gb_gemm_opts": "GemmOpts", "gb_tune_choice": "TuneChoice", "gb_gemm_desc": "GemmDesc",
           "gb_request": "Request", "gb_server_config": "ServerConfig", "gb_server_stats": "ServerStats"}


def test_struct_layouts_match_the_header(tmp_path):
    """sizeof and every member's offset of the structs the wrapper mirrors, as the C compiler
    lays them out from the header, against the ctypes layouts."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gbblas.h"', 'int main(void) {']
    for cname, pyname in STRUCTS.items():
        lines.append('    printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in getattr(gbblas, pyname)._fields_:
            lines.append('    printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ['    return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"), str(src), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    got = {}
    for line in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname, pyname in STRUCTS.items():
        cls = getattr(gbblas, pyname)
        assert got[(cname, "sizeof")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
