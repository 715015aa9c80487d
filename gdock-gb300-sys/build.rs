//! Link the prebuilt CUDA library.  `python -m gdock_gb300.build` (nvcc,
//! sm_103a) writes it to `<repo>/gdock_gb300/_build/`; GDOCK_GB300_LIB_DIR
//! overrides that directory.  The library is C ABI only: nothing here
//! compiles CUDA.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("GDOCK_GB300_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap())
            .join("..")
            .join("gdock_gb300")
            .join("_build"),
    };
    let name = if env::var("CARGO_FEATURE_DEBUG_CHECKS").is_ok() {
        "gdock_gb300_debug"
    } else {
        "gdock_gb300"
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib={}", name);
    // the shared library is found at run time from the same directory
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", dir.display());
    println!("cargo:rerun-if-env-changed=GDOCK_GB300_LIB_DIR");
    println!("cargo:rerun-if-changed=../include/gdock_gb300.h");
}
