// Links libresvg_gb300.so.  RESVG_GB300_LIB_DIR names the directory holding
// it (the package's _native/ directory after `python -m resvg_gb300.build`).
fn main() {
    println!("cargo:rerun-if-env-changed=RESVG_GB300_LIB_DIR");
    let dir = std::env::var("RESVG_GB300_LIB_DIR").unwrap_or_else(|_| {
        let here = std::env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR");
        format!("{}/../_native", here)
    });
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=resvg_gb300");
}
