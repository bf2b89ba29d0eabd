// build.rs — builds libvoxgpu.so (sm_103a) with the repository's own build step and links
// it. VOXGPU_REPO names the checkout of this repository.
use std::{env, path::PathBuf, process::Command};

fn main() {
    let repo = PathBuf::from(env::var("VOXGPU_REPO").expect("VOXGPU_REPO: path of the voxgpu repo"));
    let status = Command::new("python3")
        .current_dir(&repo)
        .args(["-c", "import __graft_entry__ as g; g.build()"])
        .status()
        .expect("python3");
    assert!(status.success(), "voxgpu build failed");
    let lib = repo.join("wgpu-voxel-engine_gb300/voxgpu");
    println!("cargo:rustc-link-search=native={}", lib.display());
    println!("cargo:rustc-link-lib=dylib=voxgpu");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib.display());
    println!("cargo:rerun-if-changed={}", repo.join("include/voxgpu.h").display());
}
