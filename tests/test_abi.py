"""The C-ABI library: it loads, exports every entry point include/misfit_gb.h
declares, and its host-side file helpers follow the reference's parse rules.
No GPU is needed for anything here."""
import os
import re

import numpy as np
import pytest

from misfit_gb300 import build, native
from tests import _golden as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.load_library()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "misfit_gb.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)  # declarations only, not comments
    return sorted(set(re.findall(r"\b(mf_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(native.EXPORTS) == syms


def test_version_and_status_strings(lib):
    assert lib.mf_version() == 10200
    assert lib.mf_status_string(0) == b"ok"
    assert lib.mf_status_string(-3) == b"malformed input file"


def test_open_without_device_fails_with_status(lib, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    g = G.load("sample")
    from misfit_gb300 import workloads as W
    p = str(tmp_path / "s.egr")
    W.write_egr(p, int(g["n"]), g["nindex"], g["nlist"])
    with pytest.raises(native.MisfitError) as e:
        native.Graph.open_egr(p)
    assert e.value.status in (-4, -1)


def test_batch_file_parse_rules(lib, tmp_path):
    p = tmp_path / "1.mtx"
    p.write_text("% comment\n1 2\n3 3\n4 5 extra\n0 7\n9 100\nx y\n6\n7 8\n  10\t2\n")
    u, v = native.read_batch_file(str(p), 20)
    # self-loop, id 0 (-> -1), id beyond n, non-numeric and short lines dropped
    assert u.tolist() == [0, 3, 6, 9]
    assert v.tolist() == [1, 4, 7, 1]


def test_mis_file_rules(lib, tmp_path):
    p = tmp_path / "mis.txt"
    p.write_text("1\n5\n5\n0\n99\n3\n")
    mis, lines = native.read_mis_file(str(p), 10)
    assert mis.tolist() == [1, 0, 1, 0, 1, 0, 0, 0, 0, 0]
    assert lines == 4  # in-range lines, duplicates included (src/misfit/misfit.cu:784-788)
    bad = tmp_path / "bad.txt"
    bad.write_text("1\nabc\n")
    with pytest.raises(native.MisfitError):
        native.read_mis_file(str(bad), 10)
    out = tmp_path / "out.txt"
    native.write_mis_file(str(out), mis)
    assert out.read_text() == "1\n3\n5\n"


def test_batch_folder_order(lib, tmp_path):
    for name in ["10.mtx", "2.mtx", "1.mtx", "3"]:
        (tmp_path / name).write_text("1 2\n")
    (tmp_path / "sub").mkdir()
    assert native.list_batch_files(str(tmp_path)) == ["1.mtx", "2.mtx", "3", "10.mtx"]
    (tmp_path / "notes.txt").write_text("x")
    with pytest.raises(native.MisfitError):
        native.list_batch_files(str(tmp_path))


def test_struct_layouts_match_the_header(tmp_path):
    """Every public struct of include/misfit_gb.h has the same size and field
    offsets in C (compiled here with the host compiler) as its ctypes mirror
    in misfit_gb300/native.py, field for field and in the same order."""
    import ctypes
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"mf_batch_stats": native.BatchStats, "mf_tuning": native.Tuning, "mf_pool_stats": native.PoolStats,
               "mf_batched_opts": native.BatchedOpts, "mf_batched_stats": native.BatchedStats}
    header = open(os.path.join(ROOT, "include", "misfit_gb.h")).read()
    lines = ['#include <stdio.h>', '#include "misfit_gb.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (cname, cname), header, flags=re.S)
        assert body, cname
        decl = re.sub(r"/\*.*?\*/", "", body.group(1), flags=re.S)
        cfields = re.findall(r"\b([a-z_][a-z_0-9]*)\s*;", decl)
        assert cfields == [f[0] for f in cls._fields_], cname   # same names, same order
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in cfields:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.split() for line in subprocess.check_output([str(exe)], text=True).splitlines())
    for cname, cls in mirrors.items():
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(cls, f).offset, (cname, f)
