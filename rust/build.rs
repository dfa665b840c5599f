//! Builds libmantaray_gpu.so from the CUDA / C++ sources of
//! mantaray_gb300/csrc with nvcc for sm_103a (the same units and flags as
//! mantaray_gb300/build.py), and links the crate against it.  With
//! $MANTARAY_GPU_LIB_DIR set, links the library found there instead.
//! Takes the place of the reference's build.rs, which only adds PyO3's link
//! arguments (that call is kept, behind the `python` feature).

use std::env;
use std::path::{Path, PathBuf};
use std::process::Command;

/// Translation units and their extra flags: the integrators without
/// implicit FMA contraction (-fmad=false), the single-scenario batched
/// builds with FP32 subnormals flushed as well.
const UNITS: &[(&str, &[&str])] = &[
    ("rk4_f64.cu", &["-fmad=false"]),
    ("api.cu", &[]),
    ("netcdf3.cpp", &[]),
    ("diag.cu", &[]),
    ("rk4_f32.cu", &["-fmad=false"]),
    ("rk4_f32_one.cu", &["-fmad=false", "-ftz=true"]),
    ("batch_api.cu", &[]),
    ("batch_static.cu", &[]),
    ("diff.cu", &[]),
    ("order.cu", &[]),
    ("seed.cu", &["-fmad=false"]),
];

fn nvcc() -> PathBuf {
    if let Ok(p) = env::var("NVCC") {
        return PathBuf::from(p);
    }
    let cuda = env::var("CUDA_HOME").unwrap_or_else(|_| "/usr/local/cuda".to_string());
    Path::new(&cuda).join("bin").join("nvcc")
}

fn run(cmd: &mut Command) {
    let status = cmd.status().unwrap_or_else(|e| panic!("cannot run {:?}: {e}", cmd));
    assert!(status.success(), "{:?} failed with {status}", cmd);
}

fn build_library(root: &Path, out: &Path) -> PathBuf {
    let csrc = root.join("mantaray_gb300").join("csrc");
    let include = root.join("include");
    let mut objects = Vec::new();
    for (unit, flags) in UNITS {
        let src = csrc.join(unit);
        println!("cargo:rerun-if-changed={}", src.display());
        let obj = out.join(format!("{unit}.o"));
        run(Command::new(nvcc())
            .args(["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                   "-lineinfo", "-Xcompiler", "-fPIC"])
            .arg("-I").arg(&include)
            .arg("-I").arg(&csrc)
            .args(*flags)
            .arg("-c").arg(&src)
            .arg("-o").arg(&obj));
        objects.push(obj);
    }
    for header in ["batch.h", "batch_handle.h", "bits.h", "fields.h", "handles.h", "k2.cuh",
                   "kernels.h", "lookup.cuh", "netcdf3.h", "ray_exact.cuh"] {
        println!("cargo:rerun-if-changed={}", csrc.join(header).display());
    }
    println!("cargo:rerun-if-changed={}", include.join("mantaray_gpu.h").display());
    run(Command::new(nvcc())
        .args(["-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o"])
        .arg(out.join("libmantaray_gpu.so"))
        .args(&objects));
    out.to_path_buf()
}

fn main() {
    #[cfg(feature = "python")]
    pyo3_build_config::add_extension_module_link_args();

    println!("cargo:rerun-if-env-changed=MANTARAY_GPU_LIB_DIR");
    let lib_dir = match env::var("MANTARAY_GPU_LIB_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => {
            let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
            let root = manifest.parent().expect("the crate sits in the repository").to_path_buf();
            build_library(&root, &PathBuf::from(env::var("OUT_DIR").unwrap()))
        }
    };
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=mantaray_gpu");
    // the extension module finds the library where it was built or found
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
}
