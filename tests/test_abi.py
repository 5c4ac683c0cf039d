"""The C-ABI library loads and exports every function its headers declare
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions(header):
    names = set()
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for m in re.finditer(r"^\s*(?:int|int32_t|size_t|void)\s+\**\s*(sgba_\w+)\s*\(", text, flags=re.M):
        names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(pkg):
    """include/sgba.h is libsgba.so's ABI, include/sgba_synth.h the scene
    generator's (libsgba_synth.so); every header in include/ is one of them."""
    assert sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")) == \
        ["sgba.h", "sgba_synth.h"]
    lib = ctypes.CDLL(pkg.native.lib_path())
    declared = _declared_functions("sgba.h")
    assert "sgba_optimize" in declared and "sgba_problem_create" in declared
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(pkg.native.EXPORTED) <= declared
    gen = ctypes.CDLL(pkg.synth.LIB_PATH)
    gen_declared = _declared_functions("sgba_synth.h")
    assert gen_declared == {"sgba_synth_generate", "sgba_synth_free"}
    assert all(hasattr(gen, n) for n in gen_declared)
    # the generator is not part of the product library
    assert not hasattr(lib, "sgba_synth_generate")


def test_abi_version_and_error_buffer(pkg):
    L = pkg.native.lib()
    assert L.sgba_abi_version() == 2
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


def _c_structs(text):
    """typedef struct { ... } name; -> [field names in order] (comments removed)."""
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = decl.strip()
            if decl:
                fields.append(re.match(r".*?(\w+)\s*(\[[^\]]*\])?$", decl, flags=re.S).group(1))
        out[m.group(2)] = fields
    return out


def _rust_structs(text):
    out = {}
    for m in re.finditer(r"pub struct (\w+)\s*\{(.*?)\n\}", text, flags=re.S):
        out[m.group(1)] = re.findall(r"^\s*pub (\w+)\s*:", m.group(2), flags=re.M)
    return out


def test_rust_ffi_declarations_match_the_header():
    """rust/sgba-sys/src/ffi.rs declares every function of include/sgba.h and
    its structs with the same fields in the same order (the crate is not
    compiled here; this keeps the declarations in step with the header)."""
    header = open(os.path.join(ROOT, "include", "sgba.h")).read()
    ffi = open(os.path.join(ROOT, "rust", "sgba-sys", "src", "ffi.rs")).read()
    c_fns = set(re.findall(r"^\s*(?:int|int32_t|size_t)\s+\**\s*(sgba_\w+)\s*\(",
                           re.sub(r"/\*.*?\*/", "", header, flags=re.S), flags=re.M))
    rust_fns = set(re.findall(r"pub fn (sgba_\w+)\s*\(", ffi))
    assert c_fns and c_fns == rust_fns, (sorted(c_fns - rust_fns), sorted(rust_fns - c_fns))
    c_structs = _c_structs(header)
    rust_structs = _rust_structs(ffi)
    for name, fields in c_structs.items():
        assert name in rust_structs, name
        assert rust_structs[name] == fields, (name, fields, rust_structs[name])


# ctypes mirrors in native.py of the header's structs
_CTYPES_OF = {"sgba_problem_desc": "ProblemDesc", "sgba_opt_params": "OptParamsC", "sgba_iter_record": "IterRecord",
              "sgba_layout": "Layout", "sgba_problem_options": "ProblemOptions", "sgba_profile": "Profile",
              "sgba_window_result": "WindowResult", "sgba_linear_solver": "LinearSolverC",
              "sgba_pcg_stats": "PcgStats", "sgba_pcg_train_params": "PcgTrainParams",
              "sgba_batch_stats": "BatchStats", "sgba_pose_graph": "PoseGraph"}


def test_python_struct_layouts_match_the_header(pkg, tmp_path):
    """sizeof and every field offset of the header's structs, as gcc lays them
    out, equal the ctypes mirrors'."""
    import subprocess
    fields = _c_structs(open(os.path.join(ROOT, "include", "sgba.h")).read())
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sgba.h"', "int main(void) {"]
    for cname in _CTYPES_OF:
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in fields[cname]:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    c = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                      text=True).stdout.splitlines())
    for cname, pyname in _CTYPES_OF.items():
        S = getattr(pkg.native, pyname)
        assert int(c[cname]) == ctypes.sizeof(S), cname
        assert [f[0] for f in S._fields_] == fields[cname], cname
        for f in fields[cname]:
            assert int(c["%s.%s" % (cname, f)]) == getattr(S, f).offset, (cname, f)


def test_camera_options_validated_without_gpu(pkg):
    """sgba_problem_create_ex rejects bad camera options on the host."""
    L = pkg.native.lib()
    h = ctypes.c_void_p()
    desc = pkg.native.ProblemDesc()
    for model, ab in ((2, (0.0, 0.0)), (-1, (0.0, 0.0)), (pkg.native.CAMERA_PINHOLE, (0.5, 1.0)),
                      (pkg.native.CAMERA_EUCM, (float("nan"), 1.0)), (pkg.native.CAMERA_EUCM, (0.5, float("inf")))):
        o = pkg.native.ProblemOptions()
        o.camera_model = model
        o.eucm_alpha_beta[0], o.eucm_alpha_beta[1] = ab
        assert L.sgba_problem_create_ex(ctypes.byref(desc), ctypes.byref(o), 0, ctypes.byref(h)) == \
            pkg.native.ERR_INVALID_ARGUMENT, (model, ab)
        assert not h.value
    o = pkg.native.ProblemOptions()
    o.intrinsics_free = 2
    assert L.sgba_problem_create_ex(ctypes.byref(desc), ctypes.byref(o), 0, ctypes.byref(h)) == \
        pkg.native.ERR_INVALID_ARGUMENT


def _c_enum_values(text):
    """NAME = value pairs of the header's enums (comments removed)."""
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(SGBA_\w+)\s*=\s*(-?\d+)", text)}


def test_enum_values_match_the_bindings(pkg):
    """The status codes, variable kinds and query modes of include/sgba.h have
    the same values in the Python and Rust bindings."""
    header = _c_enum_values(open(os.path.join(ROOT, "include", "sgba.h")).read())
    ffi = open(os.path.join(ROOT, "rust", "sgba-sys", "src", "ffi.rs")).read()
    rust = {m.group(1): int(m.group(2)) for m in re.finditer(r"pub const (SGBA_\w+): \w+ = (-?\d+);", ffi)}
    native = pkg.native
    for name, value in header.items():
        if name.startswith(("SGBA_ERR_", "SGBA_VAR_", "SGBA_QUERY_")):
            assert rust.get(name) == value, (name, value, rust.get(name))
            py = getattr(native, name[len("SGBA_"):], None)
            assert py == value, (name, value, py)
    assert header["SGBA_ERR_FACTORIZATION"] == -9 and header["SGBA_VAR_INTRINSICS"] == 0


def test_covariance_arguments_checked_without_gpu(pkg):
    """sgba_covariance_* reject a NULL problem on the host."""
    L = pkg.native.lib()
    assert L.sgba_covariance_prepare(None, None) == pkg.native.ERR_INVALID_ARGUMENT
    assert L.sgba_covariance_release(None) == pkg.native.ERR_INVALID_ARGUMENT
    assert L.sgba_covariance_blocks(None, 0, 0, None, None, None) == pkg.native.ERR_INVALID_ARGUMENT
