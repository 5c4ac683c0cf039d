"""The C-ABI library loads and exports every function its headers declare
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|int32_t|size_t|void)\s+\**\s*(sgba_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg.native.lib_path())
    declared = _declared_functions()
    assert "sgba_optimize" in declared and "sgba_problem_create" in declared
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(pkg.native.EXPORTED) <= declared


def test_abi_version_and_error_buffer(pkg):
    L = pkg.native.lib()
    assert L.sgba_abi_version() == 1
    buf = ctypes.create_string_buffer(8)
    L.sgba_last_error(buf, 8)  # no error yet or a previous one; must not overflow
    assert len(buf.value) < 8


def test_null_arguments_fail_cleanly_without_gpu(pkg):
    """Argument validation happens on the host before any CUDA call."""
    L = pkg.native.lib()
    h = ctypes.c_void_p()
    assert L.sgba_problem_create(None, 0, ctypes.byref(h)) == pkg.native.ERR_INVALID_ARGUMENT
    assert "NULL" in pkg.native.last_error()
    desc = pkg.native.ProblemDesc()
    desc.n_cam = 0
    assert L.sgba_problem_create(ctypes.byref(desc), 0, ctypes.byref(h)) == pkg.native.ERR_INVALID_ARGUMENT
    assert L.sgba_optimizer_init(None, None) == pkg.native.ERR_INVALID_ARGUMENT
