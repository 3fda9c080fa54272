// Links liblqgpu.so, built in-tree by the repository's __graft_entry__.build() into
// lattice-qcd-rs_gb300/_build (or the directory named by LQGPU_LIB_DIR).
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("LQGPU_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => {
            let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("CARGO_MANIFEST_DIR"));
            manifest.join("../../lattice-qcd-rs_gb300/_build")
        }
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=lqgpu");
    println!("cargo:rerun-if-env-changed=LQGPU_LIB_DIR");
}
