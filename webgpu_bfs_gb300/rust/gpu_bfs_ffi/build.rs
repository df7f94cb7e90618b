// Links libmsbfs.so from the directory named by MSBFS_LIB_DIR, or from the
// in-tree build folder (webgpu_bfs_gb300/_lib) next to this crate.
fn main() {
    let dir = std::env::var("MSBFS_LIB_DIR").unwrap_or_else(|_| {
        let here = std::env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR");
        format!("{here}/../../_lib")
    });
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=msbfs");
    println!("cargo:rerun-if-env-changed=MSBFS_LIB_DIR");
}
