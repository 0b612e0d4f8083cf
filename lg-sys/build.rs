// Links liblightgarden_cuda.so.  LG_LIB_DIR names the directory that holds it (the package's
// light_garden_gb300/_lib after `python -m light_garden_gb300.build`).
fn main() {
    println!("cargo:rerun-if-env-changed=LG_LIB_DIR");
    let dir = std::env::var("LG_LIB_DIR").unwrap_or_else(|_| "../light_garden_gb300/_lib".to_string());
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=lightgarden_cuda");
}
