"""The engine never routes through the oracle: no module of the package
imports it, no engine source includes or links it, and the library loader
names only the in-tree engine library (static checks, CPU)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "puncpp_gb300")


def _files(top, exts):
    for d, _, names in os.walk(top):
        if "_build" in d or "__pycache__" in d:
            continue
        for n in names:
            if n.endswith(exts):
                yield os.path.join(d, n)


def test_package_modules_do_not_import_the_oracle():
    pat = re.compile(r"^\s*(import|from)\s+[\w.]*oracle|sys\.path.*oracle|liboracle", re.M)
    bad = [p for p in _files(PKG, (".py",)) if pat.search(open(p).read())]
    assert not bad, bad


def test_engine_sources_do_not_include_or_link_the_oracle():
    pat = re.compile(r'#\s*include\s*[<"][^>"]*oracle|liboracle|oracle\.cpp', re.I)
    srcs = list(_files(os.path.join(PKG, "csrc"), (".cu", ".cuh", ".cpp", ".h"))) + \
        list(_files(os.path.join(ROOT, "include"), (".h", ".hpp")))
    assert srcs
    bad = [p for p in srcs if pat.search(open(p).read())]
    assert not bad, bad
    build = open(os.path.join(PKG, "build_lib.py")).read()
    assert "oracle" not in build


def test_loader_uses_the_in_tree_library_and_fails_loudly(tmp_path):
    import pytest
    from puncpp_gb300 import _lib
    assert os.path.dirname(os.path.abspath(_lib.LIB_PATH)) == PKG
    missing = str(tmp_path / "libpunc_gpu.so")
    saved, _lib._lib = _lib._lib, None
    try:
        with pytest.raises(FileNotFoundError):
            _lib.load(missing)
    finally:
        _lib._lib = saved
