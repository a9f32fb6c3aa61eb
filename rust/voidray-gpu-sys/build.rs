// Links libvoidray_gb300.so.  The library is built by the Python build step
// (`python -c "import __graft_entry__ as g; g.build()"`, which compiles the
// sm_103a kernels with nvcc into voidray_gb300/_lib/); point
// VOIDRAY_GB300_LIB_DIR at that folder.
fn main() {
    println!("cargo:rerun-if-env-changed=VOIDRAY_GB300_LIB_DIR");
    let dir = std::env::var("VOIDRAY_GB300_LIB_DIR")
        .unwrap_or_else(|_| concat!(env!("CARGO_MANIFEST_DIR"), "/../../voidray_gb300/_lib").to_string());
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=voidray_gb300");
}
