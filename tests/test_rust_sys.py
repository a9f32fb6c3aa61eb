"""The Rust `-sys` crate (rust/voidray-gpu-sys) against the C headers.

There is no Rust toolchain here, so the crate is not compiled; this test
reads its `src/lib.rs` as text and checks that it restates include/*.h item
for item: every struct with the same fields in the same order and the
corresponding Rust types (so the #[repr(C)] layouts are the C layouts), every
opaque handle, every function with the same argument types and return type,
and every enum value and numeric #define.  The crate is what a voidray
maintainer adds to call the library from voidray_renderer in place of
iterative_render (voidray_renderer/src/render/iterative.rs:11-16)."""
import re
from pathlib import Path

import c_header

ROOT = Path(__file__).resolve().parents[1]
LIB_RS = ROOT / "rust" / "voidray-gpu-sys" / "src" / "lib.rs"
PRIM = {"float": "f32", "double": "f64", "uint32_t": "u32", "int32_t": "i32", "uint64_t": "u64", "uint16_t": "u16",
        "uint8_t": "u8", "size_t": "usize", "char": "c_char", "void": "c_void"}


def rust_type(t, arr=0):
    base, depth, consts = t
    s = PRIM.get(base, base)
    for k in range(depth):
        s = ("*const " if consts[k] else "*mut ") + s
    return f"[{s}; {arr}]" if arr else s


def norm(t: str) -> str:
    return re.sub(r"\s+", " ", t.strip())


def read_rust():
    text = re.sub(r"//[^\n]*", "", LIB_RS.read_text())
    structs, opaque = {}, set()
    for m in re.finditer(r"#\[repr\(C\)\]\s*(?:#\[derive\([^)]*\)\]\s*)?pub struct (\w+)\s*\{(.*?)\n\}", text, re.S):
        body = m.group(2)
        if re.fullmatch(r"\s*_p: \[u8; 0\],\s*", body):
            opaque.add(m.group(1))
            continue
        structs[m.group(1)] = [(f.group(1), norm(f.group(2))) for f in re.finditer(r"pub (\w+): ([^,\n]+),", body)]
    ext = text[text.index('extern "C" {'):]
    fns = {}
    for m in re.finditer(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", ext, re.S):
        params = [norm(p.split(":", 1)[1]) for p in m.group(2).split(",") if p.strip()]
        fns[m.group(1)] = (norm(m.group(3) or "()"), params)
    consts = {m.group(1): int(m.group(2).replace("_", ""), 0) if "<<" not in m.group(2) else
              int(m.group(2).split("<<")[0]) << int(m.group(2).split("<<")[1])
              for m in re.finditer(r"pub const (\w+): \w+ = ([^;]+);", text)}
    aliases = set(re.findall(r"pub type (\w+) = i32;", text))
    return structs, opaque, fns, consts, aliases


def test_crate_files_exist():
    crate = ROOT / "rust" / "voidray-gpu-sys"
    assert (crate / "Cargo.toml").exists() and (crate / "build.rs").exists() and LIB_RS.exists()
    assert 'links = "voidray_gb300"' in (crate / "Cargo.toml").read_text()
    assert "rustc-link-lib=dylib=voidray_gb300" in (crate / "build.rs").read_text()


def test_structs_match_header_field_for_field():
    h = c_header.read(ROOT / "include")
    structs, opaque, _, _, _ = read_rust()
    assert set(structs) == set(h["structs"]), set(structs) ^ set(h["structs"])
    for name, fields in h["structs"].items():
        want = [(f, rust_type(t, arr)) for f, t, arr in fields]
        assert structs[name] == want, (name, structs[name], want)
    assert opaque == h["opaque"]


def test_functions_match_header_signature_for_signature():
    h = c_header.read(ROOT / "include")
    _, _, fns, _, aliases = read_rust()
    assert set(fns) == set(h["functions"]), set(fns) ^ set(h["functions"])
    for name, (ret, params) in h["functions"].items():
        rret, rparams = fns[name]
        assert rret == ("()" if ret[:2] == ("void", 0) else rust_type(ret)), name
        assert rparams == [rust_type(t) for _, t in params], (name, rparams)
    # the C enum types travel as i32 aliases
    assert {"vr_status", "vr_material_kind", "vr_env_kind", "vr_estimator"} <= aliases


def test_constants_match_header_values():
    h = c_header.read(ROOT / "include")
    _, _, _, consts, _ = read_rust()
    want = dict(h["defines"])
    for vals in h["enums"].values():
        want.update(vals)
    missing = {k for k in want if k not in consts}
    assert not missing, missing
    for k, v in want.items():
        assert consts[k] == v, (k, consts[k], v)
