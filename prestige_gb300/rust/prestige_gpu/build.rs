//! Compiles the CUDA library (every `.cu` file of the csrc directory) for sm_103a with nvcc
//! through the `cc` crate and links it with the CUDA runtime.  Host code is compiled without
//! floating-point contraction, as the library's own build does, so host-side constants follow
//! the oracle's operation order.
use std::env;
use std::path::PathBuf;

fn main() {
    let here = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
    let csrc = env::var("PRESTIGE_GPU_CSRC")
        .map(PathBuf::from)
        .unwrap_or_else(|_| here.join("../prestige_gb300/csrc"));
    let include = env::var("PRESTIGE_GPU_INCLUDE")
        .map(PathBuf::from)
        .unwrap_or_else(|_| here.join("../include"));

    let mut build = cc::Build::new();
    build
        .cuda(true)
        .cudart("shared")
        .flag("-gencode")
        .flag("arch=compute_103a,code=sm_103a")
        .flag("-std=c++17")
        .flag("-O3")
        .flag("-lineinfo")
        .flag("--expt-relaxed-constexpr")
        .flag("-Xcompiler")
        .flag("-ffp-contract=off")
        .flag("-Xcompiler")
        .flag("-fno-strict-aliasing")
        .include(&include)
        .include(&csrc);
    let mut sources: Vec<PathBuf> = std::fs::read_dir(&csrc)
        .expect("the CUDA sources (set PRESTIGE_GPU_CSRC)")
        .filter_map(|e| e.ok().map(|e| e.path()))
        .filter(|p| p.extension().map_or(false, |x| x == "cu"))
        .collect();
    sources.sort();
    for s in &sources {
        build.file(s);
        println!("cargo:rerun-if-changed={}", s.display());
    }
    for e in std::fs::read_dir(&csrc).unwrap().filter_map(|e| e.ok()) {
        println!("cargo:rerun-if-changed={}", e.path().display());
    }
    println!("cargo:rerun-if-changed={}", include.join("prestige_gpu.h").display());
    println!("cargo:rerun-if-env-changed=PRESTIGE_GPU_CSRC");
    println!("cargo:rerun-if-env-changed=PRESTIGE_GPU_INCLUDE");
    build.compile("prestige_gpu");

    if let Ok(cuda) = env::var("CUDA_HOME").or_else(|_| env::var("CUDA_PATH")) {
        println!("cargo:rustc-link-search=native={}/lib64", cuda);
    } else {
        println!("cargo:rustc-link-search=native=/usr/local/cuda/lib64");
    }
    println!("cargo:rustc-link-lib=dylib=cudart");
    println!("cargo:rustc-link-lib=dylib=dl");
    println!("cargo:rustc-link-lib=dylib=stdc++");
}
