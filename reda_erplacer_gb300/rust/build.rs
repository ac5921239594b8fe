// build.rs for the ERPlacer crate: link liberplacer_gb300.so (the sm_103a
// placement loop behind include/erplacer.h) into the reda-erplacer binary.
//
// The shared library is built by this repository's own recipe
// (`python -c "import __graft_entry__ as g; g.build()"`, which runs nvcc with
// -gencode arch=compute_103a,code=sm_103a) and found through
// ERPLACER_GB300_DIR.  The crate already lists `cc` as a build-dependency
// (Cargo.toml:39-40) but ships no build script; this is the one to add.
// Not built here: this environment has no Rust toolchain.
fn main() {
    let dir = std::env::var("ERPLACER_GB300_DIR")
        .expect("ERPLACER_GB300_DIR: the directory holding liberplacer_gb300.so");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=erplacer_gb300");
    // let the installed binary find the library next to where it was linked
    println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    println!("cargo:rerun-if-env-changed=ERPLACER_GB300_DIR");
}
