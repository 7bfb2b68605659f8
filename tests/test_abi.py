"""The C-ABI library loads without a GPU and exports every entry point of
include/punc_gpu.h; host-only entry points work on the CPU."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "punc_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_bindings_cover_the_header():
    from puncpp_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_abi_version(lib):
    from puncpp_gb300 import _lib
    assert lib.pg_abi_version() == _lib.ABI_VERSION == 3


def test_philox_known_answers(lib, oracle_mod):
    kat = json.load(open(os.path.join(ROOT, "tests", "golden", "philox4x32_10_kat.json")))
    for v in kat["vectors"]:
        ctr = (C.c_uint32 * 4)(*[int(x, 16) for x in v["ctr"]])
        key = (C.c_uint32 * 2)(*[int(x, 16) for x in v["key"]])
        out = (C.c_uint32 * 4)()
        assert lib.pg_philox4x32_10(ctr, key, out) == 0
        assert ["%08x" % x for x in out] == v["out"]
        out2 = (C.c_uint32 * 4)()
        oracle_mod.lib().or_philox_block(ctr, key, out2)
        assert ["%08x" % x for x in out2] == v["out"]


def test_oracle_exp_series_accuracy(oracle_mod):
    L = oracle_mod.lib()
    xs = np.concatenate([np.linspace(-740, 700, 20001), np.linspace(-40, 0, 10001), [0.0, -1e-300, 1e-300]])
    got = np.array([L.or_exp_series(float(x)) for x in xs])
    ref = np.exp(xs)
    rel = np.abs(got - ref) / np.maximum(ref, 1e-300)
    assert rel[ref > 1e-300].max() < 4e-16


def build_cpp_time_loop(tmp_path):
    """Compile tests/cpp/time_loop.cpp (a PUNC++-shaped loop on include/punc_gpu.hpp)."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = tmp_path / "time_loop"
    libdir = os.path.join(ROOT, "puncpp_gb300")
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "time_loop.cpp"), "-L" + libdir, "-lpunc_gpu",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_front_end_compiles_and_links(lib, tmp_path):
    assert build_cpp_time_loop(tmp_path).exists()


def test_errors_are_status_codes_not_aborts(lib):
    from puncpp_gb300 import _lib
    h = C.c_void_p()
    assert lib.pg_mesh_build(None, 1.0, C.byref(h)) == 1
    assert b"empty" in lib.pg_last_error()
    assert lib.pg_mesh_array(None, 0, None, None) == 1
    assert _lib.STATUS_NAMES[lib.pg_philox4x32_10(None, None, None)] == "PG_ERR_ARG"


def test_every_handle_entry_point_refuses_a_null_handle(lib):
    """Each entry point that takes an engine handle returns PG_ERR_ARG for a
    NULL handle before it touches the device (no GPU needed)."""
    from puncpp_gb300 import _lib
    scalars = (C.c_int64, C.c_int32, C.c_double, C.c_uint64, C.c_uint32, C.c_int)
    skip = {"pg_mesh_build", "pg_mesh_array", "pg_mesh_free", "pg_destroy"}
    checked = 0
    for name, (args, res) in _lib.SIGNATURES.items():
        if name in skip or not args or args[0] is not C.c_void_p:
            continue
        call = [0 if a in scalars else None for a in args]
        if res is C.c_int:
            assert getattr(lib, name)(*call) == 1, name
        else:
            assert getattr(lib, name)(*call) is None, name   # pg_stage_name
        checked += 1
    assert checked >= 40
    assert lib.pg_destroy(None) == 0


_SCALAR = {"int": "i32", "int32_t": "i32", "int64_t": "i64", "uint32_t": "u32", "uint64_t": "u64",
           "double": "f64", "char": "i8"}


def _header_prototypes():
    src = open(os.path.join(ROOT, "include", "punc_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(pg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        kinds = []
        for a in [x.strip() for x in args.split(",") if x.strip() and x.strip() != "void"]:
            is_ptr = "*" in a or "[" in a
            words = re.sub(r"\[.*?\]", "", a).replace("*", " ").replace("const", " ").split()
            base = words[0]
            kinds.append(("ptr", base) if is_ptr else ("val", _SCALAR[base]))
        protos[name] = (ret.replace("const", "").strip(), kinds)
    return protos


def _ctypes_kind(t):
    simple = {C.c_int32: "i32", C.c_int: "i32", C.c_int64: "i64", C.c_uint32: "u32", C.c_uint64: "u64",
              C.c_double: "f64", C.c_char: "i8"}
    if t in simple:
        return ("val", simple[t])
    if t in (C.c_void_p, C.c_char_p):
        return ("ptr", None if t is C.c_void_p else "char")
    target = getattr(t, "_type_", None)
    if target is C.c_void_p:
        return ("ptr", "void")       # void ** data, or an opaque handle's address (pg_sim **)
    if target in simple:
        return ("ptr", {v: k for k, v in _SCALAR.items() if k != "int"}.get(simple[target], simple[target]))
    return ("ptr", "struct")


def test_binding_argument_types_match_the_header():
    """Every ctypes signature passes each argument with the header's kind:
    the same integer width and signedness, double, or a pointer to the same
    element type (opaque handles and structures as pointers)."""
    from puncpp_gb300 import _lib
    protos = _header_prototypes()
    assert set(protos) == set(_lib.SIGNATURES)
    for name, (args, _) in _lib.SIGNATURES.items():
        ret, kinds = protos[name]
        assert len(args) == len(kinds), name
        for k, (t, (hk, hb)) in enumerate(zip(args, kinds)):
            ck, cb = _ctypes_kind(t)
            assert ck == hk, (name, k)
            if hk == "val":
                assert cb == hb, (name, k, cb, hb)
            elif cb == "void":
                assert hb == "void" or hb.startswith("pg_"), (name, k, hb)
            elif cb not in (None, "struct"):
                assert cb == hb or (cb == "int32_t" and hb == "int"), (name, k, cb, hb)
            elif cb == "struct":
                assert hb.startswith("pg_"), (name, k, hb)


_STRUCTS = {"MeshDesc": "pg_mesh_desc", "Config": "pg_config", "Object": "pg_object", "Source": "pg_source",
            "Species": "pg_species", "SolveInfo": "pg_solve_info", "StepArgs": "pg_step_args",
            "StepResult": "pg_step_result", "Tuning": "pg_tuning", "PoissonLayout": "pg_poisson_layout"}


def test_binding_structures_match_the_header_layout(tmp_path):
    """Each ctypes Structure has the size and field offsets of its C struct
    (a C program built against include/punc_gpu.h prints them)."""
    import shutil
    import subprocess
    from puncpp_gb300 import _lib
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "punc_gpu.h"', "int main(void) {"]
    expect = []
    for py, cs in _STRUCTS.items():
        cls = getattr(_lib, py)
        lines.append(f'    printf("%zu\\n", sizeof({cs}));')
        expect.append(C.sizeof(cls))
        for fname, *_ in cls._fields_:
            lines.append(f'    printf("%zu\\n", offsetof({cs}, {fname}));')
            expect.append(getattr(cls, fname).offset)
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    got = [int(x) for x in out.stdout.split()]
    assert got == expect


def test_mixed_store_is_bounded_so_deposit_sums_cannot_overflow(lib):
    """The mixed form's deposit adds q lambda in int64 units of 2^-30 q_max:
    one particle adds at most 2^30 units to a dof, so a store of at most 2^32
    slots keeps every dof's sum below 2^62 whatever the particle distribution.
    A larger store is refused with PG_ERR_CAPACITY before the device is
    touched (no GPU needed)."""
    from puncpp_gb300 import _lib as L
    from puncpp_gb300 import meshgen, punc
    fixed_bits, max_slots = 30, 1 << 32
    assert max_slots * (1 << fixed_bits) <= 1 << 62
    mesh = punc.Mesh(meshgen.kuhn_box(2))
    cfg = L.Config()
    cfg.precision = L.PG_MIXED
    cfg.particle_capacity = max_slots + 1
    h = C.c_void_p()
    rc = lib.pg_create(mesh.handle, C.byref(cfg), C.byref(h))
    assert L.STATUS_NAMES[rc] == "PG_ERR_CAPACITY" and not h.value
    msg = lib.pg_last_error()
    assert b"at most 4294967296 particle slots" in msg and b"2^-30" in msg
