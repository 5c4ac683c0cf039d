// Links libsgba.so, which the repository's build step produces with nvcc and
// g++ (`python -c "import __graft_entry__ as g; g.build()"` writes it to
// sophus-rs_gb300/libsgba.so). SGBA_LIB_DIR names the directory that holds
// it; without it the system library path is searched.
fn main() {
    println!("cargo:rerun-if-env-changed=SGBA_LIB_DIR");
    if let Ok(dir) = std::env::var("SGBA_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
        println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    }
    println!("cargo:rustc-link-lib=dylib=sgba");
}
