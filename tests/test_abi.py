"""The C ABI without a GPU: struct layouts against the C compiler, the exported symbols of
liblightgarden_cuda.so against every function ``include/lg.h`` declares, and the calls whose
behaviour is defined before any device work (argument checks, defaults, version)."""
import ctypes as C
import json
import re
import subprocess

import pytest

from light_garden_gb300 import abi

HEADER = abi.LIB_DIR.parent.parent / "include" / "lg.h"

STRUCTS = [abi.lg_geo, abi.lg_object, abi.lg_light, abi.lg_blend_component, abi.lg_mod_color, abi.lg_string_mod,
           abi.lg_params, abi.lg_segment, abi.lg_chord, abi.lg_path_record, abi.lg_trace_stats, abi.lg_device_opts, abi.lg_scene_desc,
           abi.lg_serve_opts, abi.lg_serve_step_stats]


def declared_functions():
    """Names of the functions declared in lg.h (prototypes at file scope)."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(lg_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    """sizeof / offsetof of every struct field as the C compiler lays it out."""
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', 'int main(void) {',
             'printf("{");']
    first = True
    for s in STRUCTS:
        name = s.__name__
        items = [f'"\\"{name}\\": %zu"', ] + [f'"\\"{name}.{f}\\": %zu"' for f, *_ in s._fields_]
        args = [f"sizeof({name})"] + [f"offsetof({name}, {f})" for f, *_ in s._fields_]
        for it, a in zip(items, args):
            sep = "" if first else ", "
            first = False
            lines.append(f'printf("{sep}" {it}, {a});')
    lines += ['printf("}\\n");', "return 0; }"]
    src = d / "layout.c"
    src.write_text("\n".join(lines))
    exe = d / "layout"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-o", str(exe), str(src)], check=True)
    return json.loads(subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout)


def test_header_compiles_as_c_and_cxx(tmp_path):
    for cc, ext in (("gcc", "c"), ("g++", "cpp")):
        src = tmp_path / f"h.{ext}"
        src.write_text(f'#include "{HEADER}"\nint main(void) {{ return LG_ABI_VERSION == 5 ? 0 : 1; }}\n')
        subprocess.run([cc, "-Wall", "-Werror", "-pedantic", "-o", str(tmp_path / f"h_{ext}"), str(src)],
                       check=True)


@pytest.mark.parametrize("struct", STRUCTS, ids=lambda s: s.__name__)
def test_struct_layout_matches_c(struct, c_layout):
    name = struct.__name__
    assert C.sizeof(struct) == c_layout[name], f"sizeof({name})"
    for f, *_ in struct._fields_:
        assert getattr(struct, f).offset == c_layout[f"{name}.{f}"], f"offsetof({name}, {f})"


def test_record_sizes_are_the_documented_ones():
    # one segment = 4 f32 endpoints + RGBA f32 (the reference's vertex pair, sub_render_pass.rs:188-203)
    assert C.sizeof(abi.lg_segment) == 32
    assert C.sizeof(abi.lg_path_record) == 24
    assert abi.segment_dtype().itemsize == 32 and abi.path_dtype().itemsize == 24
    # a string-mod line: two vertices with their own colours (string_mod.rs:118-119)
    assert C.sizeof(abi.lg_chord) == 48 and abi.chord_dtype().itemsize == 48


def test_every_declared_function_is_exported(cuda_lib):
    names = declared_functions()
    assert len(names) >= 15, names
    bound = {n for n, *_ in abi.EXPORTS}
    assert set(names) == bound, f"header vs bindings: {set(names) ^ bound}"
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], check=True, capture_output=True,
                         text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert getattr(cuda_lib, n) is not None


def test_library_exports_only_the_abi(cuda_lib):
    """No stray C++ or CUDA runtime symbols leak into the dynamic symbol table as lg_*."""
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], check=True, capture_output=True,
                         text=True).stdout
    lg = sorted(l.split()[-1] for l in out.splitlines() if l.split()[-1].startswith("lg_"))
    assert lg == declared_functions()


def test_abi_version_and_defaults(cuda_lib):
    assert cuda_lib.lg_abi_version() == 5
    p = abi.lg_params()
    cuda_lib.lg_params_default(C.byref(p))
    assert p.max_bounce == 5  # Tracer::new, tracer.rs:37
    assert list(p.cutoff_color) == pytest.approx([0.001] * 4)  # tracer.rs:38
    assert (p.width, p.height) == (512, 512)
    assert list(p.clear_color) == [0.0, 0.0, 0.0, 1.0]
    assert (p.color_blend.src_factor, p.color_blend.dst_factor, p.color_blend.op) == (
        abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_ADD)  # mod.rs:67-71
    assert (p.alpha_blend.src_factor, p.alpha_blend.dst_factor, p.alpha_blend.op) == (
        abi.LG_BF_SRC_ALPHA, abi.LG_BF_ONE, abi.LG_BO_ADD)
    assert p.accum == abi.LG_ACCUM_FIXED64
    assert p.precision == abi.LG_PRECISION_EXACT and (p.ray_stride, p.ray_offset) == (1, 0)
    # the Python mirror builds the same defaults
    q = abi.params_default()
    assert bytes(q) == bytes(p)
    cuda_lib.lg_params_default(None)  # tolerated


def test_null_context_is_an_argument_error(cuda_lib):
    L = cuda_lib
    s = abi.lg_trace_stats()
    assert L.lg_create(None, None) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_trace(None, C.byref(s)) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_accumulate(None, C.byref(s)) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_accumulate_segments(None, None, 0, None) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_resolve_f16(None, None, 0, 0) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_resolve_rgba8(None, None, 0, 0) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_render(None, None, 0, 0, None) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_segments_download(None, None, None, 0, None) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_accum_download(None, None, 0) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_scene_upload(None, None, 0, None, 0, None, 0, None) == abi.LG_ERR_INVALID_ARGUMENT
    assert L.lg_last_error(None) == b"null context"
    assert L.lg_destroy(None) in (abi.LG_OK, abi.LG_ERR_INVALID_ARGUMENT)


def test_create_rejects_bad_culling_options(cuda_lib):
    """Option checks come before any device work (no GPU needed)."""
    h = C.c_void_p()
    for culling, density in ((3, 0.0), (-1, 0.0), (abi.LG_CULL_ON, -1.0), (abi.LG_CULL_AUTO, float("nan"))):
        opts = abi.lg_device_opts()
        opts.culling, opts.grid_density = culling, density
        assert cuda_lib.lg_create(C.byref(h), C.byref(opts)) == abi.LG_ERR_INVALID_ARGUMENT
        assert not h.value


def test_noalloc_argument_checks_precede_device_work(cuda_lib):
    p = abi.params_default()
    n = C.c_uint64(123)
    assert cuda_lib.lg_accumulate_segments_noalloc(None, 5, C.byref(p), None, None, C.byref(n)) == \
        abi.LG_ERR_INVALID_ARGUMENT
    assert cuda_lib.lg_accumulate_segments_noalloc(None, 0, None, None, None, None) == abi.LG_ERR_INVALID_ARGUMENT


def test_create_without_a_gpu_fails_cleanly(cuda_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p(1)
    st = cuda_lib.lg_create(C.byref(h), None)
    assert st == abi.LG_ERR_CUDA
    assert not h.value


def test_python_context_has_no_cpu_fallback(monkeypatch, tmp_path):
    """Without the built library the product path raises instead of computing elsewhere."""
    monkeypatch.setattr(abi, "LIB_PATH", tmp_path / "missing.so")
    monkeypatch.setattr(abi, "_lib", None)
    from light_garden_gb300.runtime import Context
    with pytest.raises(RuntimeError, match="missing"):
        Context()


# ---- the Rust binding (lg-sys, written for hosts with a Rust toolchain; none is here) -------
RUST = abi.LIB_DIR.parent.parent / "lg-sys" / "src" / "lib.rs"
_RUST_SIZES = {"i8": 1, "u8": 1, "i16": 2, "u16": 2, "i32": 4, "u32": 4, "f32": 4, "i64": 8, "u64": 8, "f64": 8,
               "usize": 8}


def _rust_structs():
    text = re.sub(r"//[^\n]*", "", RUST.read_text())
    out = {}
    for name, body in re.findall(r"pub struct (\w+)\s*\{(.*?)\}", text, flags=re.S):
        out[name] = re.findall(r"pub (\w+):\s*([^,]+),", body)
    return out


def _rust_size(ty, structs_by_name):
    ty = ty.strip()
    m = re.fullmatch(r"\[(.+);\s*(\d+)\]", ty)
    if m:
        return _rust_size(m.group(1), structs_by_name) * int(m.group(2))
    if ty.startswith("*"):
        return 8
    if ty in _RUST_SIZES:
        return _RUST_SIZES[ty]
    return C.sizeof(structs_by_name[ty])


def test_rust_binding_matches_the_header():
    """lg-sys declares every struct with the fields, order and sizes of the ctypes mirror
    (itself checked against the C compiler above), every function of the header, and the
    same ABI version."""
    rs = _rust_structs()
    by_name = {s.__name__: s for s in STRUCTS}
    for s in STRUCTS:
        assert s.__name__ in rs, s.__name__
        fields = rs[s.__name__]
        assert [f for f, _ in fields] == [f for f, *_ in s._fields_], s.__name__
        for (f, ty), (_, cty, *_) in zip(fields, s._fields_):
            assert _rust_size(ty, by_name) == C.sizeof(cty), (s.__name__, f, ty)
    text = RUST.read_text()
    fns = set(re.findall(r"pub fn (lg_\w+)\(", text))
    assert fns == set(declared_functions())
    assert f"pub const LG_ABI_VERSION: u32 = {abi.LG_ABI_VERSION};" in text
