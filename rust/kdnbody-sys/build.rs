//! Link libkdnbody.so (built by `python -m multilanguagekdtree_gb300.build_ext`) and the CUDA
//! runtime.  KDNBODY_LIB_DIR names the directory of libkdnbody.so (default: the Python
//! package directory next to this crate); CUDA_HOME the CUDA toolkit (default /usr/local/cuda).
use std::env;
use std::path::PathBuf;

fn main() {
    let lib_dir = match env::var("KDNBODY_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("cargo sets this"))
            .join("..")
            .join("..")
            .join("multilanguagekdtree_gb300"),
    };
    let cuda = env::var("CUDA_HOME").unwrap_or_else(|_| "/usr/local/cuda".to_string());
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-search=native={}/lib64", cuda);
    println!("cargo:rustc-link-lib=dylib=kdnbody");
    println!("cargo:rustc-link-lib=dylib=cudart");
    // the shared library is found at run time next to where it was linked from
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
    println!("cargo:rerun-if-env-changed=KDNBODY_LIB_DIR");
    println!("cargo:rerun-if-env-changed=CUDA_HOME");
    println!("cargo:rerun-if-changed=build.rs");
}
