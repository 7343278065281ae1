"""The uncompiled Rust binding (rust/rayna_gpu_sys) against the C header: it
declares every entry point the header declares, and every structure's fields
in the header's order with matching widths. (No Rust toolchain in this
image: this is the check available without compiling it.)"""
import os
import re

from rayna_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SYS = os.path.join(ROOT, "rust", "rayna_gpu_sys", "src", "lib.rs")

RUST_TO_CTYPE = {"u32": "c_uint", "i32": "c_int", "u64": "c_ulong", "f32": "c_float", "f64": "c_double"}


def rust_structs(text):
    out = {}
    for m in re.finditer(r"pub struct (rg_\w+) \{(.*?)\n\}", text, flags=re.S):
        fields = re.findall(r"pub (\w+): ([^,]+),", m.group(2))
        out[m.group(1)] = [(n, t.strip()) for n, t in fields]
    return out


def test_rust_sys_declares_every_header_function():
    from test_abi_host import declared_symbols
    text = open(SYS).read()
    fns = set(re.findall(r"pub fn (rg_\w+)\(", text))
    assert fns == set(declared_symbols())
    assert "pub const RG_ABI_VERSION: u32 = 8;" in text


def test_rust_sys_struct_fields_follow_the_ctypes_mirror():
    text = open(SYS).read()
    structs = rust_structs(text)
    for name in ("rg_material", "rg_texture", "rg_volume", "rg_sdf", "rg_scene_desc", "rg_camera", "rg_render_opts",
                 "rg_render_stats", "rg_hit", "rg_scene_info", "rg_tuning", "rg_batch_tuning", "rg_gradients",
                 "rg_device_opts", "rg_image"):
        cty = getattr(A, name)
        ours = [n for n, _ in cty._fields_]
        assert [n for n, _ in structs[name]] == ours, name
        for (fname, rty), (_, cfield) in zip(structs[name], cty._fields_):
            base = rty.strip("[]; 0123456789")
            if rty.startswith("*"):
                continue
            want = RUST_TO_CTYPE.get(base.split(";")[0].strip("[ "))
            if want and hasattr(cfield, "_type_"):
                assert want in cfield._type_.__name__ or cfield._type_.__name__.startswith(want[:4]), (name, fname)
