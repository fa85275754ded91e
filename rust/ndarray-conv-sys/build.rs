// Links libndconv.so (built by ndarray-conv_gb300/build.py into
// ndarray-conv_gb300/_build/) and the CUDA runtime it was built against.
//   NDCONV_LIB_DIR  directory holding libndconv.so
//   CUDA_LIB_DIR    directory holding libcudart.so (default /usr/local/cuda/lib64)
fn main() {
    println!("cargo:rerun-if-env-changed=NDCONV_LIB_DIR");
    println!("cargo:rerun-if-env-changed=CUDA_LIB_DIR");
    if let Ok(dir) = std::env::var("NDCONV_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
    }
    let cuda = std::env::var("CUDA_LIB_DIR").unwrap_or_else(|_| "/usr/local/cuda/lib64".to_string());
    println!("cargo:rustc-link-search=native={cuda}");
    println!("cargo:rustc-link-lib=dylib=ndconv");
    println!("cargo:rustc-link-lib=dylib=cudart");
}
