// Links libomg_cuda.so. OMG_CUDA_LIB_DIR names the directory that holds it
// (omg_audio_gb300/ of a built checkout of this library).
fn main() {
    let dir = std::env::var("OMG_CUDA_LIB_DIR").unwrap_or_else(|_| "omg_audio_gb300".to_string());
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=omg_cuda");
    println!("cargo:rerun-if-env-changed=OMG_CUDA_LIB_DIR");
}
