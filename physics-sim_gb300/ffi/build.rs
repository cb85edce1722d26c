// Links libdemgb.so.  The library is built in place by
// physics-sim_gb300/build_lib.py (nvcc, sm_103a); DEMGB_LIB_DIR overrides
// where it is looked for (default: the directory above this crate).
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("DEMGB_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join(".."),
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=demgb");
    println!("cargo:rerun-if-env-changed=DEMGB_LIB_DIR");
}
