//! Link libcasars_cuda.so.  The library is built by the Python package's
//! build step (nvcc for sm_103a) into casa-rs_gb300/lib/; CASARS_CUDA_LIB_DIR
//! overrides that directory.
use std::env;
use std::path::PathBuf;

fn main() {
    println!("cargo:rerun-if-env-changed=CASARS_CUDA_LIB_DIR");
    let dir = match env::var("CASARS_CUDA_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("../../lib"),
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=casars_cuda");
    println!("cargo:rerun-if-changed=../../../include/casars_cuda.h");
}
