//! Links libcfft_gb300.so.  By default the library is built in the enclosing
//! package (concrete-fft_gb300/build.py runs nvcc for sm_103a, in parallel, no
//! cmake); CFFT_GB300_LIB_DIR points at a prebuilt copy instead.
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    println!("cargo:rerun-if-env-changed=CFFT_GB300_LIB_DIR");
    let lib_dir = match env::var("CFFT_GB300_LIB_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => {
            let pkg = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("..");
            let status = Command::new(env::var("PYTHON").unwrap_or_else(|_| "python3".into()))
                .arg(pkg.join("build.py"))
                .status()
                .expect("running concrete-fft_gb300/build.py (needs python3 and nvcc)");
            assert!(status.success(), "concrete-fft_gb300/build.py failed");
            for dir in ["csrc", "../include"] {
                println!("cargo:rerun-if-changed={}", pkg.join(dir).display());
            }
            pkg.join("lib")
        }
    };
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=cfft_gb300");
    // the library is loaded from its build directory at run time as well
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
}
