// vox_types.h — structures shared by the host code and the kernels (plain C++).
#pragma once

#include <cstdint>
#include <type_traits>

#include "voxgpu.h"

namespace vox {

constexpr unsigned ERR_TIMEOUT = 1u;   // a look-back wait gave up
constexpr unsigned ERR_CAPACITY = 2u;  // output capacity exceeded
constexpr unsigned ERR_BAD_INPUT = 4u; // a slot index, or a hashed coordinate, out of range
// set in a status mirror word by the launch that wrote it (MeshArgs::err_mirror)
constexpr unsigned kMirrorValid = 0x80000000u;

// Bounded spin: ~2^22 polls with a growing nanosleep (well under 2 s in total).
constexpr int kSpinLimit = 1 << 22;

enum GenMode : int { GM_OCC = 0, GM_HEIGHT = 1, GM_DENSITY = 2, GM_BERNOULLI = 3 };

struct GenDev {
  int kind;
  int octaves;
  unsigned long long seed;
  float freq, lac, gain, amp, base, y_ref, y_scale;
  int solid_below_zero;
};

// Per-context constant tables, computed on the host once (see vox_tables.cpp).
struct TablesDev {
  float corner[6][4][3];  // rotated quad corner offsets per emission direction
  float part[6][3][3];    // T*R entries (i<3, j<3) before the t_i * 0 term
  float row3[6][3];       // T*R row 3, columns 0..2
  float uv[4][2];         // quad::VERTICES tex coords
  uint32_t tex[6];        // texture index per emission direction
  uint32_t slot[6];       // face slot per emission direction
  uint8_t perm[512];      // noise permutation
  float grad[16][4];      // gradient coefficients (gx, gy, gz, 0) of hash & 15
};

struct BatchCtl {
  unsigned int next;       // work-queue ticket; reset to 0 by the last CTA of a launch
  unsigned int epoch;      // look-back state tag; advanced by the last CTA of a launch
  unsigned int err;        // ERR_* bits, sticky until the host clears them
  unsigned int bar_count;  // grid barrier: CTAs arrived (reset by the last arriver)
  unsigned int bar_gen;    // grid barrier: generation, advanced by the last arriver
  unsigned int scan_flag;  // phased kernel: the generation whose offset scan is complete
  unsigned int done;       // CTAs finished in a launch that mirrors its status (reset by the last)
  unsigned int pad;
};

struct MeshArgs {
  int n;
  long long index_base;
  const vox_chunk_coord* coords;
  const uint8_t* nbr_mask;
  const uint32_t* occ_pool;   // GM_OCC, batch: chunk i at occ_pool + slots[i] * words
  const int32_t* slots;
  const int32_t* nbr_slots;   // 6 per chunk, -1 = not loaded
  int pool_slots;             // number of slots in occ_pool (bounds check)
  const uint32_t* occ_self;   // GM_OCC, single chunk
  const uint32_t* occ_nbr[6];
  vox_chunk_coord coord_single;
  void* out0;
  void* out1;
  unsigned long long cap;
  unsigned long long* face_offsets;  // n + 1 entries (single chunk: the count at [0])
  unsigned long long* state;         // look-back states, n entries
  BatchCtl* ctl;
  const TablesDev* tables;
  GenDev gen;
  int full6;
  int stage_faces;                   // faces per staging window (0: direct global stores)
  int spin_limit;                    // polls before a look-back wait gives up
  uint32_t* scratch;                 // phased/overlap kernels: per-chunk spilled chunk state
  int split;                         // phased/overlap kernels: emission segments per chunk
  uint32_t* counts;                  // phased kernel: per-chunk face totals
  int lane_flush;                    // staged faces leave shared memory by plain stores
  int lag;                           // overlap kernel: generation items ahead of emission
  unsigned* err_mirror;              // page-locked host word for the launch's status, or null
  // Global face index of this launch's first face, or null for 0. A batch cut into several
  // launches (slabs) points every later launch at its own face_offsets[0], which the previous
  // launch of the same stream wrote as its total; every offset and output index of the
  // launch is shifted by it.
  const unsigned long long* base_ptr;
  // k_generate_planes: the number of listed chunks, read from device memory (at most n;
  // CTAs at or beyond it return at once).
  const unsigned* n_dev;
};

}  // namespace vox
