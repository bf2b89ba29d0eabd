// The raw binding, re-exported at the crate root.
#![allow(non_camel_case_types)]
mod voxgpu_sys;
pub use voxgpu_sys::*;
