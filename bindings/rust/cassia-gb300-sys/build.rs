// Links libcassia_gb300.so.  The library is built in-tree by the Python build
// step (cassia_gb300/_build/); set CASSIA_GB300_LIB_DIR to link elsewhere.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = env::var("CASSIA_GB300_LIB_DIR").map(PathBuf::from).unwrap_or_else(|_| {
        PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("../../../cassia_gb300/_build")
    });
    println!("cargo:rerun-if-env-changed=CASSIA_GB300_LIB_DIR");
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=cassia_gb300");
}
