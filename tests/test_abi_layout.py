"""The ctypes structures of the Python binding against the C header: a small
C program compiled with gcc prints every struct's size and each field's
offset, and the binding must agree field by field (same names, same order)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {"prx_options": "Options", "prx_result": "Result", "prx_ppr_result": "PprResult",
           "prx_tune_result": "TuneResult", "prx_ppr_tune_result": "PprTuneResult", "prx_host_csr": "HostCsr"}


@pytest.fixture(scope="module")
def layout(tmp_path_factory):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    from pagerank_gb300 import _lib
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "pagerank_gb300.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in getattr(_lib, pyname)._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    return _lib, got


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_struct_matches_header(layout, cname):
    _lib, got = layout
    cls = getattr(_lib, STRUCTS[cname])
    assert C.sizeof(cls) == got[(cname, "size")], cname
    for field, _ in cls._fields_:
        assert getattr(cls, field).offset == got[(cname, field)], (cname, field)


def test_bindings_cover_every_header_field():
    """Each struct's fields in the header, in order, are the binding's."""
    import re
    from pagerank_gb300 import _lib
    text = open(os.path.join(ROOT, "include", "pagerank_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for cname, pyname in STRUCTS.items():
        body = re.search(r"typedef struct \{([^}]*)\}\s*" + cname + ";", text).group(1)
        names = []
        for decl in body.split(";"):
            decl = decl.strip()
            if decl:
                names.append(re.match(r".*?(\w+)\s*(\[\s*\w+\s*\])?$", decl, re.S).group(1))
        assert names == [f for f, _ in getattr(_lib, pyname)._fields_], cname
