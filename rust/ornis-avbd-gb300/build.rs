//! Links libornis_avbd.so.  ORNIS_AVBD_LIB_DIR names the directory that holds
//! it (default: the in-tree build, ornis_gb300/_lib next to this crate).
fn main() {
    let dir = std::env::var("ORNIS_AVBD_LIB_DIR").unwrap_or_else(|_| {
        let here = std::env::var("CARGO_MANIFEST_DIR").unwrap();
        format!("{here}/../../ornis_gb300/_lib")
    });
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=ornis_avbd");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    println!("cargo:rerun-if-env-changed=ORNIS_AVBD_LIB_DIR");
}
