// build.rs for the film_grain crate: builds the GB300 library from its sources with nvcc (sm_103a) when
// the `gb300` feature is on, and links it.  The library's own build step (film_grain_gb300/build.py) is
// the one that knows the flags; this script runs it and points the linker at its output.
//
//   FILM_GRAIN_GB300_ROOT   checkout of this repository (default: ../film_grain_gb300 next to the crate)
//   FILM_GRAIN_GB300_LIB    directory of a prebuilt libfg_gb300.so (skips the build)
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    if env::var_os("CARGO_FEATURE_GB300").is_none() {
        return;
    }
    println!("cargo:rerun-if-env-changed=FILM_GRAIN_GB300_ROOT");
    println!("cargo:rerun-if-env-changed=FILM_GRAIN_GB300_LIB");
    let lib_dir = match env::var_os("FILM_GRAIN_GB300_LIB") {
        Some(dir) => PathBuf::from(dir),
        None => {
            let root = env::var_os("FILM_GRAIN_GB300_ROOT")
                .map(PathBuf::from)
                .unwrap_or_else(|| PathBuf::from("../film_grain_gb300"));
            println!("cargo:rerun-if-changed={}", root.join("film_grain_gb300/csrc").display());
            println!("cargo:rerun-if-changed={}", root.join("include/film_grain_gb300.h").display());
            // nvcc -gencode arch=compute_103a,code=sm_103a for every unit, then one shared library
            let status = Command::new("python3")
                .arg(root.join("film_grain_gb300/build.py"))
                .status()
                .expect("running film_grain_gb300/build.py (needs python3 and nvcc)");
            assert!(status.success(), "film_grain_gb300/build.py failed");
            root.join("film_grain_gb300/_build")
        }
    };
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=fg_gb300");
    // the library is found at run time next to the binary's rpath
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
}
