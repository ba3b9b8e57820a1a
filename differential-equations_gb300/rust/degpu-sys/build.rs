// Links the in-tree libdegpu.so; DEGPU_LIB_DIR points at differential-equations_gb300/csrc.
fn main() {
    let dir = std::env::var("DEGPU_LIB_DIR").unwrap_or_else(|_| "../../csrc".to_string());
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=degpu");
    println!("cargo:rerun-if-env-changed=DEGPU_LIB_DIR");
}
