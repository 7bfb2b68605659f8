"""The oracle's ctypes bindings (oracle/oracle.py) pass each argument of the
extern "C" functions of oracle/oracle.cpp with the definition's kind: the
checker's own boundary, checked like the engine's (CPU)."""
import os
import re

from test_abi import _SCALAR, _ctypes_kind

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _definitions():
    src = open(os.path.join(ROOT, "oracle", "oracle.cpp")).read()
    src = re.sub(r"//[^\n]*", "", src)
    out = {}
    for name, args in re.findall(r"\b(or_[a-z0-9_]+)\s*\(([^)]*)\)\s*\{", src):
        kinds = []
        for a in [x.strip() for x in args.split(",") if x.strip() and x.strip() != "void"]:
            is_ptr = "*" in a or "[" in a
            base = re.sub(r"\[.*?\]", "", a).replace("*", " ").replace("const", " ").split()[0]
            kinds.append(("ptr", base) if is_ptr else ("val", _SCALAR[base]))
        out[name] = kinds
    return out


def test_oracle_bindings_match_the_definitions(oracle_mod):
    defs = _definitions()
    assert set(oracle_mod._SIG) <= set(defs), set(oracle_mod._SIG) - set(defs)
    for name, (args, _) in oracle_mod._SIG.items():
        kinds = defs[name]
        assert len(args) == len(kinds), name
        for k, (t, (hk, hb)) in enumerate(zip(args, kinds)):
            ck, cb = _ctypes_kind(t)
            assert ck == hk, (name, k)
            if hk == "val":
                assert cb == hb, (name, k, cb, hb)
            elif cb not in (None, "struct", "void"):
                assert cb == hb or (cb == "int32_t" and hb == "int"), (name, k, cb, hb)
