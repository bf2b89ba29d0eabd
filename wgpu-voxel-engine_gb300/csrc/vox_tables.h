// vox_tables.h — host-side construction of the per-context constant tables.
#pragma once

#include "voxgpu.h"
#include "vox_types.h"

namespace vox {

// Rotation of the quad of emission direction dir (0 L, 1 R, 2 Bk, 3 F, 4 D, 5 U),
// row-major, as Quad::new computes it (src/quad.rs:14-46).
void face_rotation(int dir, float R[3][3]);

// Fills the corner/matrix/texture tables and the noise permutation for cfg.
void build_tables(const vox_config& cfg, TablesDev& t);

}  // namespace vox
