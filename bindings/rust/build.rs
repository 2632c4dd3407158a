// Links libwrach_gb300.so, built by wrach_gb300/build.py (nvcc, sm_103a).
fn main() {
    let dir = std::env::var("WRACH_GB300_LIB_DIR")
        .expect("set WRACH_GB300_LIB_DIR to the directory holding libwrach_gb300.so");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=wrach_gb300");
    println!("cargo:rerun-if-env-changed=WRACH_GB300_LIB_DIR");
}
