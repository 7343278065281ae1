// Not compiled here: this image has no Rust toolchain.
//
// Compiles the library's sources with nvcc for sm_103a (the performance
// build: device code with -fmad=true) and links the shared library built
// from them. RAYNA_GB300_ROOT points at the repository (default: two levels
// above this crate); CUDA_HOME at the toolkit (default /usr/local/cuda).
use std::env;
use std::path::PathBuf;
use std::process::Command;

const SOURCES: [&str; 6] = ["renderer.cpp", "bvh_build.cpp", "megakernel.cu", "wavefront.cu", "adjoint.cu", "batch.cu"];

fn main() {
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
    let root = env::var("RAYNA_GB300_ROOT").map(PathBuf::from).unwrap_or_else(|_| manifest.join("../.."));
    let cuda = env::var("CUDA_HOME").map(PathBuf::from).unwrap_or_else(|_| PathBuf::from("/usr/local/cuda"));
    let nvcc = cuda.join("bin/nvcc");
    let out = PathBuf::from(env::var("OUT_DIR").unwrap());
    let csrc = root.join("rayna_gb300/csrc");
    let include = root.join("include");
    let arch = ["-gencode", "arch=compute_103a,code=sm_103a"];

    // every translation unit in parallel
    let children: Vec<_> = SOURCES
        .iter()
        .map(|src| {
            let obj = out.join(format!("{}.o", src));
            let child = Command::new(&nvcc)
                .args(arch)
                .args(["-O3", "-lineinfo", "-std=c++17", "-fmad=true", "--expt-relaxed-constexpr"])
                .arg("-I").arg(&include)
                .args(["-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-c"])
                .arg(csrc.join(src))
                .arg("-o").arg(&obj)
                .spawn()
                .expect("failed to start nvcc");
            (obj, child)
        })
        .collect();
    let mut objs = Vec::new();
    for (obj, mut child) in children {
        assert!(child.wait().expect("nvcc").success(), "nvcc failed for {}", obj.display());
        objs.push(obj);
    }
    let lib = out.join("librayna_gpu.so");
    let status = Command::new(&nvcc)
        .args(arch)
        .args(["-shared", "-cudart", "shared", "-o"])
        .arg(&lib)
        .args(&objs)
        .arg("-L").arg(cuda.join("lib64"))
        .status()
        .expect("nvcc link");
    assert!(status.success(), "link of librayna_gpu.so failed");

    println!("cargo:rustc-link-search=native={}", out.display());
    println!("cargo:rustc-link-search=native={}", cuda.join("lib64").display());
    println!("cargo:rustc-link-lib=dylib=rayna_gpu");
    println!("cargo:rustc-link-lib=dylib=cudart");
    println!("cargo:rerun-if-changed={}", include.join("rayna_gpu.h").display());
    for src in SOURCES {
        println!("cargo:rerun-if-changed={}", csrc.join(src).display());
    }
}
