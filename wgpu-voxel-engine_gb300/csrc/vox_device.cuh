// vox_device.cuh — device code of the chunk generation + meshing path (sm_103a).
//
// One CTA owns one chunk at a time. The chunk's occupancy lives in shared memory as
// one N-bit row per (y, z) (bit x = voxel solid), plus six halo rows per side. Face
// masks of a row come from shifts of the row and its neighbours, counts from popc.
// A deterministic block scan over rows gives every row's first face, the rows that have
// faces and the voxels that have faces. Chunks of a batch get their global first face
// from a decoupled look-back over a device work queue (k_mesh_batch), from one scan
// behind a grid barrier (k_mesh_batch_phased), or from a look-back over totals published
// by separate generation items (k_mesh_batch_overlap). Each warp compacts the faces of a
// run of voxels, stages them 32 at a time in shared memory in their final byte layout,
// and sends each batch to global memory with a TMA bulk copy
// (cp.async.bulk.global.shared::cta), or stores them directly.
//
// Reference semantics restated here (Blatko1/wgpu-voxel-engine):
//   fill rule            src/chunk.rs:35-45     (solid -> GRASS, else AIR)
//   culling/emission     src/chunk.rs:59-245    (y -> z -> x order; L R Bk F D U per voxel;
//                                               lateral halo only; y borders always emitted)
//   face records         src/quad.rs:14-54      (T * R instance matrix, texture index)
//   vertex expansion     src/shaders/vertex.vert:22-27
//
// Compiled with -fmad=false: every float expression rounds once per operation in the
// written order, which is what makes the noise and vertex bits match the CPU oracle.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "voxgpu.h"
#include "vox_schedule.h"
#include "vox_types.h"

namespace vox {

template <int N>
struct Shape {
  using RowT = typename std::conditional<(N > 32), unsigned long long, uint32_t>::type;
  static constexpr int R = N * N;                 // rows per chunk
  static constexpr int W = N > 32 ? N / 32 : 1;   // u32 words per row
  // CTA sizes the kernels are instantiated for (rows split evenly over the threads)
  static constexpr int T0 = N == 8 ? 32 : (N == 16 ? 128 : (N == 32 ? 256 : 512));
  static constexpr int T1 = 2 * T0;
  static constexpr int LOG2N = N == 8 ? 3 : (N == 16 ? 4 : (N == 32 ? 5 : 6));
  // Capacity of the face-voxel list (voxels with at least one face, as (row << LOG2N) | x
  // in 16 bits); a chunk with more face voxels is emitted row by row instead.
  static constexpr int VCap = N > 32 ? 0 : (N * N * N < 8192 ? N * N * N : 8192);
};

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

// Per-octave lattice data of one column coordinate (heightmap generation).
struct AxisX {
  int px, px1;  // p[X], p[X + 1]
  float fr, u;  // fractional coordinate and its fade
};
struct AxisZ {
  int y;        // lattice Y & 255
  float fr, v;  // fractional coordinate and its fade
  int pad;
};

// Octaves whose per-axis lattice data are computed between one pair of barriers.
constexpr int kOctGroup = 8;

// Density generation from per-chunk lattice tables (see dens_tables): per octave and axis
// the lattice data of the N + 2 coordinates (local -1..N), and the gradient coefficients
// of every lattice corner the chunk's coordinates touch. Configurations beyond these
// limits (more octaves, more corners, frequencies <= 0) take the per-sample hash path.
struct DensAxis {
  int ci;                  // lattice cell relative to the chunk's first cell on this axis
  float fr, fade, fr1;     // fractional coordinate, its fade, fractional - 1
};
constexpr int kDensMaxOct = 4;
template <int N>
__host__ __device__ constexpr int dens_max_corners() { return N <= 8 ? 128 : (N <= 16 ? 256 : 1024); }
// Byte offsets of the density tables in the generation scratch: int hdr[16] (per octave:
// corner-table base, corners along y and along z), DensAxis axes[octave][axis][N + 2],
// for 32^3 chunks the packed x and y records of the lane = z path (two 16-byte records
// per octave and coordinate), then the corner-pair records: record i holds the gradients
// of corner i and of corner i + 1 (its +z neighbour on the lattice) as
// {gx_i, gx_i+1, gy_i, gy_i+1} and {gz_i, gz_i+1}.
template <int N>
struct DensPlan {
  static constexpr bool kLaneZ = N == 32;
  static constexpr int kAxes = 64;
  static constexpr int kPackX = kAxes + kDensMaxOct * 3 * (N + 2) * 16;
  static constexpr int kPackY = kPackX + (kLaneZ ? kDensMaxOct * (N + 2) * 32 : 0);
  static constexpr int kPairXY = kPackY + (kLaneZ ? kDensMaxOct * (N + 2) * 32 : 0);
  static constexpr int kPairZ = kPairXY + dens_max_corners<N>() * 16;
  static constexpr int kBytes = kPairZ + dens_max_corners<N>() * 8;
};
template <int N>
__host__ __device__ constexpr int dens_scratch_bytes() {
  return DensPlan<N>::kBytes;
}
// A warp's face list: the faces of one group of 32 voxels (6 each) after fewer than one
// batch of faces carried over from the previous group.
constexpr int kWarpFaces = 32 * 6 + 32;
// Faces one warp stages at a time (each warp has two staging buffers of this many faces).
constexpr int kWarpBatch = 32;
// Bytes of one warp staging buffer (vertex records, then the index records shifted by up
// to 8 bytes; or instance records shifted by up to 12 bytes).
template <int LAYOUT>
__host__ __device__ constexpr int warp_buf_bytes() {
  return LAYOUT == VOX_LAYOUT_INSTANCED ? align16(kWarpBatch * 68 + 16)
                                        : kWarpBatch * 96 + align16(kWarpBatch * 24 + 16);
}

// Shared-memory carve-up; the same functions size the launch on the host.
template <int N, int LAYOUT>
struct SmemPlan {
  using RowT = typename Shape<N>::RowT;
  static constexpr int kTables = align16((int)sizeof(TablesDev));
  static constexpr int kOcc = align16(Shape<N>::R * (int)sizeof(RowT));
  static constexpr int kHalo = align16(6 * N * (int)sizeof(RowT));
  static constexpr int kRows = align16((Shape<N>::R + 1) * 4);
  static constexpr int kNz = align16(Shape<N>::R * 2);
  static constexpr int kVList = align16(Shape<N>::VCap * 2);
  static constexpr int kMisc = 64;
  static constexpr int kFixed0 = kTables + kOcc + kHalo + kRows + kNz + kVList + kMisc;
  // the chunk state from occ through misc (contiguous in shared memory), as spilled by the
  // phased and overlap kernels: occupancy, halo, row offsets, row and voxel lists, counts
  static constexpr int kSpill = kOcc + kHalo + kRows + kNz + kVList + kMisc;
  // per-warp face lists (face-parallel emission)
  __host__ __device__ static int list_bytes(int threads) { return (threads / 32) * kWarpFaces * 4; }
  __host__ __device__ static int fixed(int threads) { return kFixed0 + list_bytes(threads); }
  // generation scratch, aliased with the staging window
  static constexpr int kColK = align16((N + 2) * (N + 2) * 4);
  static constexpr int kAxisHalf = kOctGroup * align16((N + 2) * 16);
  static constexpr int kAxis = 2 * kAxisHalf;
  // heightmap corner tables: per-octave header, then the gradient coefficients (gx, gy)
  static constexpr int kHHdr = align16((4 * kOctGroup + 1) * 4);
  static constexpr int kHeight = kColK + kAxis + kHHdr + dens_max_corners<N>() * 8;
  static constexpr int kGenScratch =
      kHeight > dens_scratch_bytes<N>() ? kHeight : dens_scratch_bytes<N>();
  // staging area: stage_faces / kWarpBatch buffers per warp when staging (stage_faces
  // 32 or 64), else only the generation scratch
  __host__ __device__ static int stage_bytes(int threads, int stage_faces) {
    const int b = stage_faces > 0
                      ? (threads / 32) * (stage_faces / kWarpBatch) * warp_buf_bytes<LAYOUT>()
                      : 0;
    return b < kGenScratch ? kGenScratch : b;
  }
  __host__ __device__ static int total(int threads, int stage_faces) {
    return fixed(threads) + stage_bytes(threads, stage_faces);
  }
};

// ------------------------------------------------------------------------------------
// Noise (Perlin improved noise, 2002) — same operation order as the CPU oracle.
// ------------------------------------------------------------------------------------

__device__ __forceinline__ float d_fade(float t) {
  return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f);
}
__device__ __forceinline__ float d_lerp(float t, float a, float b) { return a + t * (b - a); }

// Packed FP32 pairs: one f32x2 instruction performs the operation on both halves, each
// rounded to nearest like the scalar add / sub / mul, so a pair of scalar expressions
// evaluated this way gives the same bits with half the instructions. The low half is the
// first element.
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2_pack(float lo, float hi) {
  f2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b) {
  f2_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b) {
  f2_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
  f2_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// d_lerp on both halves
__device__ __forceinline__ f2_t f2_lerp(f2_t t, f2_t a, f2_t b) {
  return f2_add(a, f2_mul(t, f2_sub(b, a)));
}
// Gradient dot products from the coefficient table (gx, gy, gz) of hash & 15.
__device__ __forceinline__ float d_grad3(const float4* gt, int h, float x, float y, float z) {
  const float4 g = gt[h & 15];
  return (g.x * x + g.y * y) + g.z * z;
}
__device__ __forceinline__ float d_grad2(const float4* gt, int h, float x, float y) {
  const float4 g = gt[h & 15];
  return g.x * x + g.y * y;
}

__device__ __forceinline__ float d_noise3(const uint8_t* p, const float4* gt, float x, float y,
                                          float z) {
  float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  float u = d_fade(x), v = d_fade(y), w = d_fade(z);
  int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
  int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
  float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float l00 = d_lerp(u, d_grad3(gt, p[AA], x, y, z), d_grad3(gt, p[BA], x1, y, z));
  float l10 = d_lerp(u, d_grad3(gt, p[AB], x, y1, z), d_grad3(gt, p[BB], x1, y1, z));
  float l01 = d_lerp(u, d_grad3(gt, p[AA + 1], x, y, z1), d_grad3(gt, p[BA + 1], x1, y, z1));
  float l11 = d_lerp(u, d_grad3(gt, p[AB + 1], x, y1, z1), d_grad3(gt, p[BB + 1], x1, y1, z1));
  return d_lerp(w, d_lerp(v, l00, l10), d_lerp(v, l01, l11));
}

// noise2 at a column whose per-axis lattice data were computed once per octave; the
// operations are those of the oracle's or_noise2_f32, minus the shared subexpressions.
__device__ __forceinline__ float d_noise2_axes(const uint8_t* p, const float4* gt, const AxisX& ax,
                                               const AxisZ& az) {
  const int A = ax.px + az.y, B = ax.px1 + az.y;
  const float x = ax.fr, y = az.fr;
  const float x1 = x - 1.0f, y1 = y - 1.0f;
  const float l0 = d_lerp(ax.u, d_grad2(gt, p[p[A]], x, y), d_grad2(gt, p[p[B]], x1, y));
  const float l1 =
      d_lerp(ax.u, d_grad2(gt, p[p[A + 1]], x, y1), d_grad2(gt, p[p[B + 1]], x1, y1));
  return d_lerp(az.v, l0, l1);
}

__device__ __forceinline__ float d_fbm3(const uint8_t* p, const float4* gt, float x, float y,
                                        float z, const GenDev& g) {
  float sum = 0.0f, amp = 1.0f, f = g.freq;
  for (int o = 0; o < g.octaves; ++o) {
    sum = sum + amp * d_noise3(p, gt, x * f, y * f, z * f);
    f = f * g.lac;
    amp = amp * g.gain;
  }
  return sum;
}

// Draw i (0-based) of splitmix64 seeded with s0 is mix(s0 + (i + 1) * gamma).
__device__ __forceinline__ unsigned long long d_splitmix_at(unsigned long long s0,
                                                            unsigned long long i) {
  unsigned long long z = s0 + (i + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// ------------------------------------------------------------------------------------
// Small helpers
// ------------------------------------------------------------------------------------

__device__ __forceinline__ int popc_row(uint32_t v) { return __popc(v); }
__device__ __forceinline__ int popc_row(unsigned long long v) { return __popcll(v); }

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// TMA bulk copies shared -> global (cp.async.bulk, bulk-group completion).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(ssrc);
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
               ::"l"(gdst), "r"(s), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
// Issues [src, src + bytes) -> dst in pieces of at most 32 KiB (16-byte multiples).
__device__ __forceinline__ void bulk_s2g_pieces(unsigned char* dst, const unsigned char* src,
                                                uint32_t bytes) {
  while (bytes > 0) {
    const uint32_t b = bytes > 32768u ? 32768u : bytes;
    bulk_s2g(dst, src, b);
    dst += b;
    src += b;
    bytes -= b;
  }
}

// Look-back state word: epoch (24 bits) | flag (2 bits) | value (38 bits).
constexpr unsigned long long kFlagAgg = 1ull;
constexpr unsigned long long kFlagIncl = 2ull;
__device__ __forceinline__ unsigned long long pack_state(unsigned epoch, unsigned long long flag,
                                                         unsigned long long value) {
  return ((unsigned long long)(epoch & 0xFFFFFFu) << 40) | (flag << 38) |
         (value & ((1ull << 38) - 1));
}

// ------------------------------------------------------------------------------------
// Shared-memory view of one chunk
// ------------------------------------------------------------------------------------

template <int N, int LAYOUT>
struct ChunkSmem {
  using RowT = typename Shape<N>::RowT;
  TablesDev* tab;
  RowT* occ;        // [R]
  RowT* halo;       // [6][N]: 0 -x (bits z, by y), 1 +x, 2 -z (bits x, by y), 3 +z, 4 -y (bits x, by z), 5 +y
  uint32_t* rows;   // [R + 1] exclusive face offsets per row
  uint16_t* nz;     // rows that have faces, ascending
  uint16_t* vlist;  // face voxels in emission order, (row << LOG2N) | x (Shape<N>::VCap)
  int* misc;        // [0] rows with faces; [1] face voxels listed in vlist, or -1
  uint32_t* lists;  // per-warp face lists (packed x, y, z, dir)
  unsigned char* stage;
  // generation scratch (aliased with the staging window)
  int* colk;        // heightmap column thresholds
  AxisX* ax;        // per-octave x-axis lattice data, [kOctGroup][N + 2]
  AxisZ* az;        // per-octave z-axis lattice data, [kOctGroup][N + 2]
  int* hhdr;        // heightmap corner tables: per octave base, corners along z, first x, first z;
                    // [4 * kOctGroup] = corner count, or -1 when the tables are not used
  float2* hcorner;  // heightmap corner gradient coefficients (gx, gy)

  __device__ void carve(unsigned char* base) {
    using P = SmemPlan<N, LAYOUT>;
    unsigned char* q = base;
    tab = reinterpret_cast<TablesDev*>(q);
    q += P::kTables;
    occ = reinterpret_cast<RowT*>(q);
    q += P::kOcc;
    halo = reinterpret_cast<RowT*>(q);
    q += P::kHalo;
    rows = reinterpret_cast<uint32_t*>(q);
    q += P::kRows;
    nz = reinterpret_cast<uint16_t*>(q);
    q += P::kNz;
    vlist = reinterpret_cast<uint16_t*>(q);
    q += P::kVList;
    misc = reinterpret_cast<int*>(q);
    q += P::kMisc;
    lists = reinterpret_cast<uint32_t*>(q);
    q += P::list_bytes(blockDim.x);
    stage = q;
    colk = reinterpret_cast<int*>(q);
    ax = reinterpret_cast<AxisX*>(q + P::kColK);
    az = reinterpret_cast<AxisZ*>(q + P::kColK + P::kAxisHalf);
    hhdr = reinterpret_cast<int*>(q + P::kColK + P::kAxis);
    hcorner = reinterpret_cast<float2*>(q + P::kColK + P::kAxis + P::kHHdr);
  }
};

template <int N, int LAYOUT>
__device__ __forceinline__ void load_tables(ChunkSmem<N, LAYOUT>& s, const TablesDev* g) {
  const int words = (int)sizeof(TablesDev) / 4;
  const uint32_t* src = reinterpret_cast<const uint32_t*>(g);
  uint32_t* dst = reinterpret_cast<uint32_t*>(s.tab);
  for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}

// Write one ballot word for the element run [e0, e0 + 32) of a row-major bit array
// whose rows are N bits wide, into 32-bit word storage `words` (row r, word r*W + x/32).
template <int N>
__device__ __forceinline__ void store_ballot(uint32_t* words, int e, bool pred) {
  const unsigned b = __ballot_sync(0xffffffffu, pred);
  const int x = e % N;
  if ((x & 31) == 0) {
    const int row = e / N;
    constexpr uint32_t kMask = N >= 32 ? 0xFFFFFFFFu : ((1u << (N & 31)) - 1u);
    const uint32_t v = N >= 32 ? b : ((b >> (threadIdx.x & 31)) & kMask);
    words[row * Shape<N>::W + (x >> 5)] = v;
  }
}

template <int N>
__device__ __forceinline__ typename Shape<N>::RowT full_row() {
  using RowT = typename Shape<N>::RowT;
  return N >= 64 ? (RowT)~0ull : (RowT)((1ull << (N & 63)) - 1ull);
}

// ------------------------------------------------------------------------------------
// Occupancy generation into shared memory
// ------------------------------------------------------------------------------------

// Halo element (h, a, b) -> local voxel coordinates (may be -1 or N).
template <int N>
__device__ __forceinline__ void halo_coord(int h, int a, int b, int& x, int& y, int& z) {
  switch (h) {
    case 0: x = -1; y = a; z = b; break;
    case 1: x = N; y = a; z = b; break;
    case 2: x = b; y = a; z = -1; break;
    case 3: x = b; y = a; z = N; break;
    case 4: x = b; y = -1; z = a; break;
    default: x = b; y = N; z = a; break;
  }
}

// Threshold of one column (local x, z in -1..N), computed by the calling lane alone: the
// fBm of the per-column path (d_noise2_axes with the lattice data of this column), then
// k = ceil(base + amp * fbm) - oy clamped to [-1, N + 1] (-1 for NaN), so that voxel
// (x, y, z) is solid iff y < k. The same operations, in the same order, as the shared-table
// path below and as the oracle.
template <int N, int LAYOUT>
__device__ __forceinline__ int column_k(const ChunkSmem<N, LAYOUT>& s, const GenDev& g, int ox,
                                        int oy, int oz, int x, int z) {
  const uint8_t* p = s.tab->perm;
  const float4* gt = reinterpret_cast<const float4*>(s.tab->grad);
  float f = g.freq, amp = 1.0f, sum = 0.0f;
  for (int o = 0; o < g.octaves; ++o) {
    const float cx = (float)(ox + x) * f, cz = (float)(oz + z) * f;
    const float flx = floorf(cx), flz = floorf(cz);
    const int lx = (int)flx & 255;
    AxisX ax;
    ax.px = p[lx];
    ax.px1 = p[lx + 1];
    ax.fr = cx - flx;
    ax.u = d_fade(ax.fr);
    AxisZ az;
    az.y = (int)flz & 255;
    az.fr = cz - flz;
    az.v = d_fade(az.fr);
    az.pad = 0;
    sum = sum + amp * d_noise2_axes(p, gt, ax, az);
    f = f * g.lac;
    amp = amp * g.gain;
  }
  const float h = g.base + g.amp * sum;
  const float cl = ceilf(h);
  long long kk = (long long)cl - (long long)oy;
  if (!(cl == cl)) kk = -1;
  return (int)(kk < -1 ? -1 : (kk > N + 1 ? N + 1 : kk));
}

// Heightmap chunk. Column thresholds colk[(z+1)*(N+2) + (x+1)] = ceil(h(x, z)) - oy,
// clamped to [-1, N + 1], so that voxel (x, y, z), y in [-1, N], is solid iff
// y < colk (the same as (float)(oy + y) < h for the integer y). The fBm runs octave by
// octave: the lattice data of every x and z coordinate are computed once per octave,
// each thread accumulating its own columns in registers.
//
// Two ways to the thresholds. The direct path (chunks up to 32^3): every lane of the row
// phase below computes the threshold of its own column itself, with no shared lattice data,
// so generation needs no CTA barrier before the row ballots. The shared-table path (larger
// chunks): the lattice data and corner tables are built once per octave in shared memory,
// every thread accumulates its columns, and the thresholds go through s.colk.
template <int N, int LAYOUT, int T>
__device__ void gen_heightmap(ChunkSmem<N, LAYOUT>& s, const GenDev& g, int ox, int oy, int oz,
                              unsigned halo_mask, bool with_halo) {
  using RowT = typename Shape<N>::RowT;
  constexpr int side = N + 2;
  constexpr bool direct = N <= 32;
  const int t = threadIdx.x;
  if (!direct) {
    constexpr int CPT = (side * side + T - 1) / T;
    const uint8_t* p = s.tab->perm;
    const float4* gt = reinterpret_cast<const float4*>(s.tab->grad);
    float acc[CPT];
  #pragma unroll
    for (int c = 0; c < CPT; ++c) acc[c] = 0.0f;
    // Corner tables (one octave group, positive frequencies, few enough corners): per octave
    // the gradient coefficients of every lattice corner the chunk's columns touch. A corner's
    // hash p[p[p[X] + Y]] depends only on its coordinates mod 256 (the permutation table is
    // doubled), so a column reads 4 table entries instead of 8 permutation bytes and 4
    // gradient entries; the arithmetic is the per-column path's, in the same order.
    bool tab = false;
    if (g.octaves <= kOctGroup) {
      if (t < 32) {
        constexpr int kCap = dens_max_corners<N>();
        int cnt = 0, ncz = 0, x0 = 0, z0 = 0;
        bool ok = true;
        if (t < g.octaves) {
          float fo = g.freq;
          for (int q = 0; q < t; ++q) fo = fo * g.lac;
          // positive, and small enough that every cell index fits an int
          ok = fo > 0.0f && fabsf((float)(ox - 1) * fo) < 1.0e9f &&
               fabsf((float)(ox + N) * fo) < 1.0e9f && fabsf((float)(oz - 1) * fo) < 1.0e9f &&
               fabsf((float)(oz + N) * fo) < 1.0e9f;
          if (ok) {
            // coordinates grow with the local index (fo > 0): local -1 has the first cell
            x0 = (int)floorf((float)(ox - 1) * fo);
            z0 = (int)floorf((float)(oz - 1) * fo);
            const int ncx = (int)floorf((float)(ox + N) * fo) - x0 + 2;
            ncz = (int)floorf((float)(oz + N) * fo) - z0 + 2;
            ok = ncx > 0 && ncz > 0 && ncx <= kCap && ncz <= kCap && ncx * ncz <= kCap;
            cnt = ok ? ncx * ncz : 0;
          }
        }
        int incl = cnt;
  #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const int u = __shfl_up_sync(0xffffffffu, incl, off);
          if (t >= off) incl += u;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const bool all_ok = __all_sync(0xffffffffu, ok);
        if (t < g.octaves) {
          s.hhdr[4 * t + 0] = incl - cnt;
          s.hhdr[4 * t + 1] = ncz;
          s.hhdr[4 * t + 2] = x0;
          s.hhdr[4 * t + 3] = z0;
        }
        if (t == 0) s.hhdr[4 * kOctGroup] = all_ok && total <= kCap ? total : -1;
      }
      __syncthreads();
      tab = s.hhdr[4 * kOctGroup] >= 0;
    }
    float f = g.freq, amp = 1.0f;
    for (int o0 = 0; o0 < g.octaves; o0 += kOctGroup) {
      const int no = g.octaves - o0 < kOctGroup ? g.octaves - o0 : kOctGroup;
      // lattice data of every x and z coordinate for the octaves [o0, o0 + no)
      for (int i = t; i < 2 * side * no; i += T) {
        const int o = i / (2 * side), r = i % (2 * side);
        const int a = r / side, k = r % side - 1;
        float fo = f;
        for (int q = 0; q < o; ++q) fo = fo * g.lac;
        const float c = (float)(a == 0 ? ox + k : oz + k) * fo;
        const float fl = floorf(c);
        const int L = (int)fl & 255;
        const float fr = c - fl;
        if (a == 0) {
          AxisX v;
          // tables: the cell relative to the table's first x; else p[X], p[X + 1]
          v.px = tab ? (int)fl - s.hhdr[4 * o + 2] : p[L];
          v.px1 = tab ? 0 : p[L + 1];
          v.fr = fr;
          v.u = d_fade(fr);
          s.ax[o * side + k + 1] = v;
        } else {
          AxisZ v;
          v.y = tab ? (int)fl - s.hhdr[4 * o + 3] : L;
          v.fr = fr;
          v.v = d_fade(fr);
          v.pad = 0;
          s.az[o * side + k + 1] = v;
        }
      }
      if (tab) {
        const int total = s.hhdr[4 * kOctGroup];
        for (int i = t; i < total; i += T) {
          int o = 0;
          for (int q = 1; q < no; ++q)
            if (i >= s.hhdr[4 * q]) o = q;
          const int jj = i - s.hhdr[4 * o], nz = s.hhdr[4 * o + 1];
          const int X = (s.hhdr[4 * o + 2] + jj / nz) & 255, Y = (s.hhdr[4 * o + 3] + jj % nz) & 255;
          const float4 gg = gt[p[p[p[X] + Y]] & 15];
          s.hcorner[i] = make_float2(gg.x, gg.y);
        }
      }
      __syncthreads();
  #pragma unroll
      for (int c = 0; c < CPT; ++c) {
        const int j = t + c * T;
        if (j < side * side) {
          const int zi = j / side, xi = j % side;
          const bool corner = (zi == 0 || zi == side - 1) && (xi == 0 || xi == side - 1);
          if (!corner) {
            float a = amp, sum = acc[c];
            if (tab) {
              for (int o = 0; o < no; ++o) {
                const AxisX ax = s.ax[o * side + xi];
                const AxisZ az = s.az[o * side + zi];
                const int nz = s.hhdr[4 * o + 1];
                const float2* C = s.hcorner + s.hhdr[4 * o] + ax.px * nz + az.y;
                const float2 g00 = C[0], g01 = C[1], g10 = C[nz], g11 = C[nz + 1];
                const float x = ax.fr, y = az.fr;
                const float x1 = x - 1.0f, y1 = y - 1.0f;
                const float l0 = d_lerp(ax.u, g00.x * x + g00.y * y, g10.x * x1 + g10.y * y);
                const float l1 = d_lerp(ax.u, g01.x * x + g01.y * y1, g11.x * x1 + g11.y * y1);
                sum = sum + a * d_lerp(az.v, l0, l1);
                a = a * g.gain;
              }
            } else {
              for (int o = 0; o < no; ++o) {
                sum = sum + a * d_noise2_axes(p, gt, s.ax[o * side + xi], s.az[o * side + zi]);
                a = a * g.gain;
              }
            }
            acc[c] = sum;
          }
        }
      }
      for (int o = 0; o < no; ++o) {
        f = f * g.lac;
        amp = amp * g.gain;
      }
      // the next group rewrites the lattice data; after the last group the thresholds
      // below use only this thread's sums
      if (o0 + kOctGroup < g.octaves) __syncthreads();
    }
  #pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const int j = t + c * T;
      if (j < side * side) {
        const float h = g.base + g.amp * acc[c];
        const float cl = ceilf(h);
        long long kk = (long long)cl - (long long)oy;
        if (!(cl == cl)) kk = -1;
        s.colk[j] = (int)(kk < -1 ? -1 : (kk > N + 1 ? N + 1 : kk));
      }
    }
    __syncthreads();
  }  // !direct
  // Rows from the column thresholds, one warp task per group of columns: the own rows of
  // a group of z values (and their -y / +y halo rows), or one lateral halo strip. Lanes
  // hold one column's threshold k each; rows below the group's smallest k are full, rows
  // at or above its largest k are empty, and the rows in between are ballots of y < k.
  {
    constexpr int G = N >= 32 ? 1 : 32 / N;  // z values per own-row task
    constexpr int S = N > 32 ? N / 32 : 1;   // 32-bit words per row
    constexpr int LW = N >= 32 ? 32 : N;     // lanes per row word
    constexpr int W = Shape<N>::W;
    constexpr uint32_t kWordFull = N >= 32 ? 0xFFFFFFFFu : ((1u << (N & 31)) - 1u);
    constexpr int kOwnTasks = (N / G) * S;
    const int lane = t & 31, warp = t >> 5;
    constexpr int nwarps = T / 32;
    uint32_t* occw = reinterpret_cast<uint32_t*>(s.occ);
    uint32_t* halow = reinterpret_cast<uint32_t*>(s.halo);
    const int sub = lane / LW, b = lane % LW;  // row word group and bit of this lane
    for (int task = warp; task < kOwnTasks + 4 * S; task += nwarps) {
      const bool own = task < kOwnTasks;
      const int h = own ? -1 : (task - kOwnTasks) / S;
      const int seg = own ? task % S : (task - kOwnTasks) % S;
      const int xb = seg * 32 + b;  // bit position within the row
      int k;
      bool active = true;  // lanes past the end of a short halo strip hold no column
      uint32_t* base;      // word of row a of the task's first row group: base[a * rstride]
      int rstride;
      if (own) {
        const int z = (task / S) * G + sub;
        k = direct ? column_k<N, LAYOUT>(s, g, ox, oy, oz, xb, z) : s.colk[(z + 1) * side + xb + 1];
        base = occw + (task / S) * G * W + seg;
        rstride = N * W;
      } else {
        // lateral halo h: row a = y, bit = position along the strip
        const int c = sub == 0 ? xb : -1;
        active = c >= 0;
        const bool used = ((halo_mask >> h) & 1u) && with_halo;
        if (c < 0 || !used) {
          k = -1;
        } else if (direct) {
          const int hx = h == 0 ? -1 : (h == 1 ? N : c), hz = h == 2 ? -1 : (h == 3 ? N : c);
          k = column_k<N, LAYOUT>(s, g, ox, oy, oz, hx, hz);
        } else if (h == 0) {
          k = s.colk[(c + 1) * side];
        } else if (h == 1) {
          k = s.colk[(c + 1) * side + N + 1];
        } else if (h == 2) {
          k = s.colk[c + 1];
        } else {
          k = s.colk[(N + 1) * side + c + 1];
        }
        base = halow + h * N * W + seg;
        rstride = W;
      }
      const int kmin = __reduce_min_sync(0xffffffffu, active ? k : N + 1);
      const int kmax = __reduce_max_sync(0xffffffffu, active ? k : -1);
      // trivial rows (own tasks: G rows of each y; halo tasks: one row of each y)
      const int gw = own ? G : 1;
      for (int j = lane; j < N * gw; j += 32) {
        const int y = j / gw, zz = j % gw;
        base[y * rstride + zz * W] = y < kmin ? kWordFull : 0u;
      }
      __syncwarp();
      const int y0 = kmin < 0 ? 0 : kmin, y1 = kmax > N ? N : kmax;
      for (int y = y0; y < y1; ++y) {
        const uint32_t bal = __ballot_sync(0xffffffffu, y < k);
        if (b == 0 && (own || sub == 0))
          base[y * rstride + sub * W] = N >= 32 ? bal : ((bal >> lane) & kWordFull);
      }
      if (own) {
        // -y and +y halo rows of these z values (bits x): y = -1 and y = N
        const bool use4 = with_halo && ((halo_mask >> 4) & 1u);
        const bool use5 = with_halo && ((halo_mask >> 5) & 1u);
        const uint32_t b4 = __ballot_sync(0xffffffffu, use4 && -1 < k);
        const uint32_t b5 = __ballot_sync(0xffffffffu, use5 && N < k);
        if (b == 0 && with_halo) {
          const int z = (task / S) * G + sub;
          halow[(4 * N + z) * W + seg] = N >= 32 ? b4 : ((b4 >> lane) & kWordFull);
          halow[(5 * N + z) * W + seg] = N >= 32 ? b5 : ((b5 >> lane) & kWordFull);
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
}

template <int N, int GM, int LAYOUT>
__device__ __forceinline__ bool gen_solid(const ChunkSmem<N, LAYOUT>& s, const GenDev& g, int x,
                                          int y, int z, int ox, int oy, int oz,
                                          unsigned long long s0) {
  if (GM == GM_DENSITY) {
    const int wy = oy + y;
    const float f = d_fbm3(s.tab->perm, reinterpret_cast<const float4*>(s.tab->grad),
                           (float)(ox + x), (float)wy, (float)(oz + z), g);
    const float d = f - ((float)wy - g.y_ref) * g.y_scale;
    return g.solid_below_zero ? (d < 0.0f) : (d > 0.0f);
  } else {  // GM_BERNOULLI
    const unsigned long long i = (unsigned long long)(x + N * z + N * N * y);
    return (d_splitmix_at(s0, i) & 1ull) != 0ull;
  }
}

// Builds the density lattice tables of a chunk in the generation scratch (all threads; ends
// with a barrier) and returns true, or returns false without a barrier when the
// configuration is beyond the table limits (the same answer in every thread). The layout
// is DensPlan's.
template <int N, int LAYOUT, int T>
__device__ bool dens_tables(ChunkSmem<N, LAYOUT>& s, const GenDev& g, int ox, int oy, int oz) {
  using P = DensPlan<N>;
  if (g.octaves > kDensMaxOct) return false;
  int* hdr = reinterpret_cast<int*>(s.stage);
  DensAxis* axes = reinterpret_cast<DensAxis*>(s.stage + P::kAxes);
  uint4* pair_xy = reinterpret_cast<uint4*>(s.stage + P::kPairXY);
  uint2* pair_z = reinterpret_cast<uint2*>(s.stage + P::kPairZ);
  const int org[3] = {ox, oy, oz};
  // corner counts (every thread computes them; cheap)
  int lo[kDensMaxOct][3], nc[kDensMaxOct][3], base[kDensMaxOct];
  int total = 0;
  float f = g.freq;
#pragma unroll
  for (int o = 0; o < kDensMaxOct; ++o) {
    if (o < g.octaves) {
      if (!(f > 0.0f)) return false;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        // coordinates grow with the local index (f > 0): local -1 has the first cell, N the last
        const int c0 = (int)floorf((float)(org[a] - 1) * f);
        const int c1 = (int)floorf((float)(org[a] + N) * f);
        lo[o][a] = c0;
        nc[o][a] = c1 - c0 + 2;  // corners along this axis
      }
      base[o] = total;
      total += nc[o][0] * nc[o][1] * nc[o][2];
      f = f * g.lac;
    }
  }
  if (total > dens_max_corners<N>()) return false;
  const int t = threadIdx.x;
  if (t < g.octaves) {
    hdr[4 * t + 0] = base[t];
    hdr[4 * t + 1] = nc[t][1];
    hdr[4 * t + 2] = nc[t][2];
  }
  // axis data: the oracle's per-sample operations, once per coordinate
  for (int i = t; i < g.octaves * 3 * (N + 2); i += T) {
    const int o = i / (3 * (N + 2)), r = i % (3 * (N + 2));
    const int a = r / (N + 2), k = r % (N + 2);
    float fo = g.freq;
    for (int q = 0; q < o; ++q) fo = fo * g.lac;
    const float c = (float)(org[a] + k - 1) * fo;
    const float fl = floorf(c);
    DensAxis v;
    v.fr = c - fl;
    v.fade = d_fade(v.fr);
    v.fr1 = v.fr - 1.0f;
    int c0 = 0, n1 = 0, n2 = 0;
#pragma unroll
    for (int q = 0; q < kDensMaxOct; ++q) {
#pragma unroll
      for (int b = 0; b < 3; ++b)
        if (q == o && b == a) c0 = lo[q][b];
      if (q == o) {
        n1 = nc[q][1];
        n2 = nc[q][2];
      }
    }
    v.ci = (int)fl - c0;
    axes[i] = v;
    if (P::kLaneZ && a < 2) {
      // packed x (a = 0) or y (a = 1) record of the lane = z path: {fr, fr, fr1, fr1} and
      // {fade, fade, offset of cell ci, offset of cell ci + 1} in corner-record units
      const int stride = a == 0 ? n1 * n2 : n2;
      uint4* rec = reinterpret_cast<uint4*>(s.stage + (a == 0 ? P::kPackX : P::kPackY)) +
                   2 * (o * (N + 2) + k);
      rec[0] = make_uint4(__float_as_uint(v.fr), __float_as_uint(v.fr), __float_as_uint(v.fr1),
                          __float_as_uint(v.fr1));
      rec[1] = make_uint4(__float_as_uint(v.fade), __float_as_uint(v.fade),
                          (unsigned)(v.ci * stride), (unsigned)((v.ci + 1) * stride));
    }
  }
  // corner gradients: hash p[p[p[X] + Y] + Z] of the corner's lattice coordinates mod 256
  // (the doubled permutation makes this the hash the per-sample chain computes)
  const uint8_t* p = s.tab->perm;
  const float4* gt = reinterpret_cast<const float4*>(s.tab->grad);
  for (int i = t; i < total; i += T) {
    int o = 0;
#pragma unroll
    for (int q = 1; q < kDensMaxOct; ++q)
      if (q < g.octaves && i >= base[q]) o = q;
    int ix = 0, iy = 0, iz = 0, l0 = 0, l1 = 0, l2 = 0, n1 = 1, n2 = 1, b0 = 0;
#pragma unroll
    for (int q = 0; q < kDensMaxOct; ++q)
      if (q == o) {
        b0 = base[q];
        n1 = nc[q][1];
        n2 = nc[q][2];
        l0 = lo[q][0];
        l1 = lo[q][1];
        l2 = lo[q][2];
      }
    const int j = i - b0;
    iz = j % n2;
    iy = (j / n2) % n1;
    ix = j / (n1 * n2);
    const int X = (l0 + ix) & 255, Y = (l1 + iy) & 255, Z = (l2 + iz) & 255;
    // corner i and its +z neighbour (the record of a chunk's last z corner is never read)
    const float4 g0 = gt[p[p[p[X] + Y] + Z] & 15];
    const float4 g1 = gt[p[p[p[X] + Y] + ((Z + 1) & 255)] & 15];
    pair_xy[i] = make_uint4(__float_as_uint(g0.x), __float_as_uint(g1.x), __float_as_uint(g0.y),
                            __float_as_uint(g1.y));
    pair_z[i] = make_uint2(__float_as_uint(g0.z), __float_as_uint(g1.z));
  }
  __syncthreads();
  return true;
}

// Density test of local sample (x, y, z), -1 <= x, y, z <= N, from the lattice tables:
// the operations of the per-sample path (d_fbm3 + the density rule), in the same order.
template <int N, int LAYOUT>
__device__ __forceinline__ bool dens_solid_tab(const ChunkSmem<N, LAYOUT>& s, const GenDev& g,
                                               int x, int y, int z, int oy) {
  using P = DensPlan<N>;
  const int* hdr = reinterpret_cast<const int*>(s.stage);
  const DensAxis* axes = reinterpret_cast<const DensAxis*>(s.stage + P::kAxes);
  const float4* pair_xy = reinterpret_cast<const float4*>(s.stage + P::kPairXY);
  const float2* pair_z = reinterpret_cast<const float2*>(s.stage + P::kPairZ);
  float sum = 0.0f, amp = 1.0f;
  for (int o = 0; o < g.octaves; ++o) {
    const DensAxis* ao = axes + o * 3 * (N + 2);
    const DensAxis ax = ao[x + 1], ay = ao[(N + 2) + y + 1], az = ao[2 * (N + 2) + z + 1];
    const int n1 = hdr[4 * o + 1], n2 = hdr[4 * o + 2];
    const int sx = n1 * n2;
    // the pair records of the four (x, y) corner columns: corners z and z + 1
    const int c = hdr[4 * o] + (ax.ci * n1 + ay.ci) * n2 + az.ci;
    const float4 q00 = pair_xy[c], q10 = pair_xy[c + sx], q01 = pair_xy[c + n2],
                 q11 = pair_xy[c + sx + n2];
    const float2 h00 = pair_z[c], h10 = pair_z[c + sx], h01 = pair_z[c + n2],
                 h11 = pair_z[c + sx + n2];
    const float3 g000 = make_float3(q00.x, q00.z, h00.x), g001 = make_float3(q00.y, q00.w, h00.y);
    const float3 g100 = make_float3(q10.x, q10.z, h10.x), g101 = make_float3(q10.y, q10.w, h10.y);
    const float3 g010 = make_float3(q01.x, q01.z, h01.x), g011 = make_float3(q01.y, q01.w, h01.y);
    const float3 g110 = make_float3(q11.x, q11.z, h11.x), g111 = make_float3(q11.y, q11.w, h11.y);
    const float xf = ax.fr, yf = ay.fr, zf = az.fr, x1 = ax.fr1, y1 = ay.fr1, z1 = az.fr1;
    const float u = ax.fade, v = ay.fade, w = az.fade;
    const float l00 = d_lerp(u, (g000.x * xf + g000.y * yf) + g000.z * zf,
                             (g100.x * x1 + g100.y * yf) + g100.z * zf);
    const float l10 = d_lerp(u, (g010.x * xf + g010.y * y1) + g010.z * zf,
                             (g110.x * x1 + g110.y * y1) + g110.z * zf);
    const float l01 = d_lerp(u, (g001.x * xf + g001.y * yf) + g001.z * z1,
                             (g101.x * x1 + g101.y * yf) + g101.z * z1);
    const float l11 = d_lerp(u, (g011.x * xf + g011.y * y1) + g011.z * z1,
                             (g111.x * x1 + g111.y * y1) + g111.z * z1);
    const float n = d_lerp(w, d_lerp(v, l00, l10), d_lerp(v, l01, l11));
    sum = sum + amp * n;
    amp = amp * g.gain;
  }
  const int wy = oy + y;
  const float d = sum - ((float)wy - g.y_ref) * g.y_scale;
  return g.solid_below_zero ? (d < 0.0f) : (d > 0.0f);
}

// The own rows of a 32^3 density chunk from the lattice tables with lane = z: a warp takes
// one y at a time, lane z testing the samples (x, y, z) of its row (y, z) and gathering
// their bits in a register, so no ballot is needed. The samples of a row are taken in blocks
// of kDensXB x coordinates, octave by octave, each keeping its fBm sum in a register (the
// per-sample sums see the same operations in the same order as octave-inner loops would).
// Within an octave the lattice cell along x changes rarely (every 1 / frequency voxels), so
// the four corner-pair records the lane's samples read — columns x0 and x0 + 1 at y0 and
// y0 + 1, each the gradients of corners z and z + 1 — stay in registers until it does, with
// the products g.y * y and g.z * z, which do not depend on x, computed once per load. The two
// corners of a record are evaluated together as f32x2 pairs: the eight gradient dot
// products as four pairs, the four x lerps as two, the two y lerps as one, then the z lerp of
// the pair's halves. Every value is the result of the operations of dens_solid_tab, in the
// same order.
constexpr int kDensXB = 8;
template <int N, int LAYOUT>
__device__ __forceinline__ void dens_rows_lane_z(ChunkSmem<N, LAYOUT>& s, const GenDev& g, int oy) {
  static_assert(N == 32 && N % kDensXB == 0, "lane = z needs 32-voxel rows");
  using P = DensPlan<N>;
  const int* hdr = reinterpret_cast<const int*>(s.stage);
  const DensAxis* axes = reinterpret_cast<const DensAxis*>(s.stage + P::kAxes);
  const ulonglong2* pack_x = reinterpret_cast<const ulonglong2*>(s.stage + P::kPackX);
  const ulonglong2* pack_y = reinterpret_cast<const ulonglong2*>(s.stage + P::kPackY);
  const ulonglong2* pair_xy = reinterpret_cast<const ulonglong2*>(s.stage + P::kPairXY);
  const f2_t* pair_z = reinterpret_cast<const f2_t*>(s.stage + P::kPairZ);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t* occw = reinterpret_cast<uint32_t*>(s.occ);
  for (int y = warp; y < N; y += nwarps) {
    const float ty = ((float)(oy + y) - g.y_ref) * g.y_scale;
    uint32_t row = 0u;
#pragma unroll 1
    for (int xs = 0; xs < N; xs += kDensXB) {
      float sum[kDensXB];
#pragma unroll
      for (int i = 0; i < kDensXB; ++i) sum[i] = 0.0f;
      float amp = 1.0f;
#pragma unroll 1
      for (int o = 0; o < g.octaves; ++o) {
        const DensAxis az = axes[o * 3 * (N + 2) + 2 * (N + 2) + lane + 1];
        const ulonglong2 ya = pack_y[2 * (o * (N + 2) + y + 1)];      // {yf, yf} {yf-1, yf-1}
        const ulonglong2 yb = pack_y[2 * (o * (N + 2) + y + 1) + 1];  // {v, v} {y0, y1 offsets}
        const f2_t zz = f2_pack(az.fr, az.fr1);
        const int zo = hdr[4 * o] + az.ci;
        const int ry0 = zo + (int)(unsigned)yb.y, ry1 = zo + (int)(unsigned)(yb.y >> 32);
        const ulonglong2* px = pack_x + 2 * (o * (N + 2) + xs + 1);
        int cur = -1;  // x offset of the records held (offsets are >= 0)
        f2_t gx00 = 0, gx10 = 0, gx01 = 0, gx11 = 0;  // {gx} of columns (x0|x1, y0|y1)
        f2_t py00 = 0, py10 = 0, py01 = 0, py11 = 0;  // {gy * y}
        f2_t pz00 = 0, pz10 = 0, pz01 = 0, pz11 = 0;  // {gz * zf, gz' * (zf - 1)}
#pragma unroll
        for (int i = 0; i < kDensXB; ++i) {
          const ulonglong2 xa = px[2 * i];      // {xf, xf} {xf-1, xf-1}
          const ulonglong2 xb = px[2 * i + 1];  // {u, u} {x0, x1 offsets}
          const int c0 = (int)(unsigned)xb.y;
          if (c0 != cur) {  // the same in every lane
            cur = c0;
            const int c1 = (int)(unsigned)(xb.y >> 32);
            const ulonglong2 q00 = pair_xy[c0 + ry0], q10 = pair_xy[c1 + ry0];
            const ulonglong2 q01 = pair_xy[c0 + ry1], q11 = pair_xy[c1 + ry1];
            gx00 = q00.x, gx10 = q10.x, gx01 = q01.x, gx11 = q11.x;
            py00 = f2_mul(q00.y, ya.x), py10 = f2_mul(q10.y, ya.x);
            py01 = f2_mul(q01.y, ya.y), py11 = f2_mul(q11.y, ya.y);
            pz00 = f2_mul(pair_z[c0 + ry0], zz), pz10 = f2_mul(pair_z[c1 + ry0], zz);
            pz01 = f2_mul(pair_z[c0 + ry1], zz), pz11 = f2_mul(pair_z[c1 + ry1], zz);
          }
          // (g.x * x + g.y * y) + g.z * z of corners (x_, y_, z) and (x_, y_, z + 1)
          const f2_t d00 = f2_add(f2_add(f2_mul(gx00, xa.x), py00), pz00);
          const f2_t d10 = f2_add(f2_add(f2_mul(gx10, xa.y), py10), pz10);
          const f2_t d01 = f2_add(f2_add(f2_mul(gx01, xa.x), py01), pz01);
          const f2_t d11 = f2_add(f2_add(f2_mul(gx11, xa.y), py11), pz11);
          const f2_t l0 = f2_lerp(xb.x, d00, d10);  // {l00, l01}
          const f2_t l1 = f2_lerp(xb.x, d01, d11);  // {l10, l11}
          float m0, m1;
          f2_unpack(f2_lerp(yb.x, l0, l1), m0, m1);
          sum[i] = sum[i] + amp * d_lerp(az.fade, m0, m1);
        }
        amp = amp * g.gain;
      }
#pragma unroll
      for (int i = 0; i < kDensXB; ++i) {
        const float d = sum[i] - ty;
        const bool solid = g.solid_below_zero ? (d < 0.0f) : (d > 0.0f);
        row |= (uint32_t)solid << (xs + i);
      }
    }
    occw[y * N + lane] = row;
  }
}

// One lateral halo plane of a 32^3 density chunk (h = 0..3: x = -1, x = N, z = -1, z = N)
// from the lattice tables, evaluated like the own rows: lane b is the sample's z (x planes)
// or x (z planes), a warp takes a contiguous run of RB rows y, octave by octave, with the
// run's sums in registers, and the four corner-pair records stay in registers while the y
// lattice cell is unchanged, with g.x * x and g.z * z computed once per load. Row y of the
// plane is the ballot over the lanes. Every value is the result of the operations of
// dens_solid_tab, in the same order.
template <int N, int LAYOUT, int RB>
__device__ __forceinline__ void dens_halo_plane_pairs(ChunkSmem<N, LAYOUT>& s, const GenDev& g, int oy,
                                                      int h) {
  static_assert(N == 32, "one sample per lane along the plane");
  using P = DensPlan<N>;
  const int* hdr = reinterpret_cast<const int*>(s.stage);
  const DensAxis* axes = reinterpret_cast<const DensAxis*>(s.stage + P::kAxes);
  const ulonglong2* pack_x = reinterpret_cast<const ulonglong2*>(s.stage + P::kPackX);
  const ulonglong2* pack_y = reinterpret_cast<const ulonglong2*>(s.stage + P::kPackY);
  const ulonglong2* pair_xy = reinterpret_cast<const ulonglong2*>(s.stage + P::kPairXY);
  const f2_t* pair_z = reinterpret_cast<const f2_t*>(s.stage + P::kPairZ);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int y0 = warp * RB;
  const int fixed = (h & 1) ? N + 1 : 0;  // table index of -1 or N
  const int xi = h < 2 ? fixed : lane + 1, zi = h < 2 ? lane + 1 : fixed;
  float sum[RB];
#pragma unroll
  for (int i = 0; i < RB; ++i) sum[i] = 0.0f;
  float amp = 1.0f;
#pragma unroll 1
  for (int o = 0; o < g.octaves; ++o) {
    const ulonglong2 xa = pack_x[2 * (o * (N + 2) + xi)];      // {xf, xf} {xf-1, xf-1}
    const ulonglong2 xb = pack_x[2 * (o * (N + 2) + xi) + 1];  // {u, u} {x0, x1 offsets}
    const DensAxis az = axes[o * 3 * (N + 2) + 2 * (N + 2) + zi];
    const f2_t zz = f2_pack(az.fr, az.fr1);
    const int zo = hdr[4 * o] + az.ci;
    const int c0 = zo + (int)(unsigned)xb.y, c1 = zo + (int)(unsigned)(xb.y >> 32);
    int cur = -1;  // y offset of the records held (offsets are >= 0)
    f2_t gy00 = 0, gy10 = 0, gy01 = 0, gy11 = 0;  // {gy} of columns (x0|x1, y0|y1)
    f2_t px00 = 0, px10 = 0, px01 = 0, px11 = 0;  // {gx * x}
    f2_t pz00 = 0, pz10 = 0, pz01 = 0, pz11 = 0;  // {gz * zf, gz' * (zf - 1)}
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      const int y = y0 + i;
      const ulonglong2 ya = pack_y[2 * (o * (N + 2) + y + 1)];      // {yf, yf} {yf-1, yf-1}
      const ulonglong2 yb = pack_y[2 * (o * (N + 2) + y + 1) + 1];  // {v, v} {y0, y1 offsets}
      const int r0 = (int)(unsigned)yb.y;
      if (r0 != cur) {  // the same in every lane
        cur = r0;
        const int r1 = (int)(unsigned)(yb.y >> 32);
        const ulonglong2 q00 = pair_xy[c0 + r0], q10 = pair_xy[c1 + r0];
        const ulonglong2 q01 = pair_xy[c0 + r1], q11 = pair_xy[c1 + r1];
        gy00 = q00.y, gy10 = q10.y, gy01 = q01.y, gy11 = q11.y;
        px00 = f2_mul(q00.x, xa.x), px10 = f2_mul(q10.x, xa.y);
        px01 = f2_mul(q01.x, xa.x), px11 = f2_mul(q11.x, xa.y);
        pz00 = f2_mul(pair_z[c0 + r0], zz), pz10 = f2_mul(pair_z[c1 + r0], zz);
        pz01 = f2_mul(pair_z[c0 + r1], zz), pz11 = f2_mul(pair_z[c1 + r1], zz);
      }
      // (g.x * x + g.y * y) + g.z * z of corners (x_, y_, z) and (x_, y_, z + 1)
      const f2_t d00 = f2_add(f2_add(px00, f2_mul(gy00, ya.x)), pz00);
      const f2_t d10 = f2_add(f2_add(px10, f2_mul(gy10, ya.x)), pz10);
      const f2_t d01 = f2_add(f2_add(px01, f2_mul(gy01, ya.y)), pz01);
      const f2_t d11 = f2_add(f2_add(px11, f2_mul(gy11, ya.y)), pz11);
      const f2_t l0 = f2_lerp(xb.x, d00, d10);  // {l00, l01}
      const f2_t l1 = f2_lerp(xb.x, d01, d11);  // {l10, l11}
      float m0, m1;
      f2_unpack(f2_lerp(yb.x, l0, l1), m0, m1);
      sum[i] = sum[i] + amp * d_lerp(az.fade, m0, m1);
    }
    amp = amp * g.gain;
  }
  uint32_t* halow = reinterpret_cast<uint32_t*>(s.halo);
#pragma unroll
  for (int i = 0; i < RB; ++i) {
    const int y = y0 + i;
    const float d = sum[i] - ((float)(oy + y) - g.y_ref) * g.y_scale;
    const unsigned b = __ballot_sync(0xffffffffu, g.solid_below_zero ? (d < 0.0f) : (d > 0.0f));
    if (lane == 0) halow[h * N + y] = b;
  }
}

// Fills s.occ (own rows) and, for every set bit of `halo_mask`, the halo rows; the other
// halo rows are zero (a neighbour that is not loaded counts as air, chunk.rs:102-107).
template <int N, int GM, int LAYOUT, int T>
__device__ void gen_chunk(ChunkSmem<N, LAYOUT>& s, const GenDev& g, vox_chunk_coord c,
                          long long chunk_index, unsigned halo_mask, bool with_halo) {
  using RowT = typename Shape<N>::RowT;
  const int ox = c.x * N, oy = c.y * N, oz = c.z * N;
  if (GM == GM_HEIGHT) {
    gen_heightmap<N, LAYOUT, T>(s, g, ox, oy, oz, halo_mask, with_halo);
    return;
  }
  const unsigned long long s0 = g.seed ^ (unsigned long long)chunk_index;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t* occw = reinterpret_cast<uint32_t*>(s.occ);
  const bool tab = GM == GM_DENSITY && dens_tables<N, LAYOUT, T>(s, g, ox, oy, oz);
  if (N == 32 && tab) {
    if constexpr (N == 32) dens_rows_lane_z<N, LAYOUT>(s, g, oy);
  } else {
    for (int base = warp * 32; base < N * N * N; base += nwarps * 32) {
      const int e = base + lane;
      const int row = e / N, x = e % N;
      const int y = row / N, z = row % N;
      store_ballot<N>(occw, e, tab ? dens_solid_tab<N, LAYOUT>(s, g, x, y, z, oy)
                                   : gen_solid<N, GM, LAYOUT>(s, g, x, y, z, ox, oy, oz, s0));
    }
  }
  if (with_halo) {
    uint32_t* halow = reinterpret_cast<uint32_t*>(s.halo);
    for (int h = 0; h < 6; ++h) {
      if ((halo_mask >> h) & 1u) {
        if constexpr (N == 32 && T >= 128) {  // N * 32 / T rows per warp
          if (tab && h < 4) {  // lateral planes of the table path: corner pairs
            dens_halo_plane_pairs<N, LAYOUT, N * 32 / T>(s, g, oy, h);
            continue;
          }
        }
        for (int base = warp * 32; base < N * N; base += nwarps * 32) {
          const int e = base + lane;
          int x, y, z;
          halo_coord<N>(h, e / N, e % N, x, y, z);
          store_ballot<N>(halow + h * N * Shape<N>::W, e,
                          tab ? dens_solid_tab<N, LAYOUT>(s, g, x, y, z, oy)
                              : gen_solid<N, GM, LAYOUT>(s, g, x, y, z, ox, oy, oz, s0));
        }
      } else {
        for (int i = threadIdx.x; i < N; i += blockDim.x) s.halo[h * N + i] = (RowT)0;
      }
    }
  }
  __syncthreads();
}

// Occupancy from global memory: own rows copied; halo rows taken from the neighbours'
// boundary planes (nbr[d] == nullptr: not loaded, zero halo).
template <int N, int LAYOUT>
__device__ void load_chunk(ChunkSmem<N, LAYOUT>& s, const uint32_t* self,
                           const uint32_t* const nbr[6], unsigned use_mask) {
  using RowT = typename Shape<N>::RowT;
  constexpr int W = Shape<N>::W;
  uint32_t* occw = reinterpret_cast<uint32_t*>(s.occ);
  for (int i = threadIdx.x; i < N * N * W; i += blockDim.x) occw[i] = __ldg(self + i);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t* halow = reinterpret_cast<uint32_t*>(s.halo);
  for (int h = 0; h < 6; ++h) {
    const uint32_t* nb = ((use_mask >> h) & 1u) ? nbr[h] : nullptr;
    if (!nb) {
      for (int i = threadIdx.x; i < N; i += blockDim.x) s.halo[h * N + i] = (RowT)0;
      continue;
    }
    if (h <= 1) {
      // bit (N-1) (h = 0) or bit 0 (h = 1) of the neighbour's row (y, z), gathered over z.
      const int bx = h == 0 ? N - 1 : 0;
      for (int base = warp * 32; base < N * N; base += nwarps * 32) {
        const int e = base + lane;
        const int y = e / N, z = e % N;
        const uint32_t w = __ldg(nb + (y * N + z) * W + (bx >> 5));
        store_ballot<N>(halow + h * N * W, e, ((w >> (bx & 31)) & 1u) != 0u);
      }
    } else {
      // whole rows: -z: (y, N-1); +z: (y, 0); -y: (N-1, z); +y: (0, z).
      for (int i = threadIdx.x; i < N * W; i += blockDim.x) {
        const int a = i / W, w = i % W;
        int r;
        if (h == 2) r = a * N + (N - 1);
        else if (h == 3) r = a * N;
        else if (h == 4) r = (N - 1) * N + a;
        else r = a;
        halow[(h * N + a) * W + w] = __ldg(nb + r * W + w);
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------------
// Face masks, counts and emission
// ------------------------------------------------------------------------------------

template <int N, int LAYOUT>
__device__ __forceinline__ void row_masks(const ChunkSmem<N, LAYOUT>& s, int y, int z,
                                          typename Shape<N>::RowT m[6]) {
  using RowT = typename Shape<N>::RowT;
  const RowT row = s.occ[y * N + z];
  const RowT lb = (s.halo[0 * N + y] >> z) & (RowT)1;
  const RowT rb = (s.halo[1 * N + y] >> z) & (RowT)1;
  const RowT ln = (row << 1) | lb;
  const RowT rn = (row >> 1) | (rb << (N - 1));
  const RowT bn = z > 0 ? s.occ[y * N + z - 1] : s.halo[2 * N + y];
  const RowT fn = z < N - 1 ? s.occ[y * N + z + 1] : s.halo[3 * N + y];
  const RowT dn = y > 0 ? s.occ[(y - 1) * N + z] : s.halo[4 * N + z];
  const RowT un = y < N - 1 ? s.occ[(y + 1) * N + z] : s.halo[5 * N + z];
  m[0] = row & ~ln;
  m[1] = row & ~rn;
  m[2] = row & ~bn;
  m[3] = row & ~fn;
  m[4] = row & ~dn;
  m[5] = row & ~un;
}

// Per-row face counts -> exclusive offsets in s.rows[0..R], the ascending list of the
// rows with faces in s.nz (count in s.misc[0]) and, when they fit, the face voxels in
// emission order in s.vlist (count in s.misc[1], else -1); returns the chunk's face total.
template <int N, int LAYOUT, int T>
__device__ uint32_t count_and_scan(ChunkSmem<N, LAYOUT>& s) {
  using RowT = typename Shape<N>::RowT;
  constexpr int RPT = Shape<N>::R / T;
  constexpr int VCap = Shape<N>::VCap;
  static_assert(RPT >= 1 && RPT * T == Shape<N>::R, "rows must split evenly over threads");
  const int t = threadIdx.x;
  uint32_t cnt[RPT];
  RowT any[RPT];
  uint32_t local = 0, vl = 0, nzl = 0;
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = t * RPT + k;
    RowT m[6];
    row_masks<N, LAYOUT>(s, r / N, r % N, m);
    uint32_t c = 0;
#pragma unroll
    for (int d = 0; d < 6; ++d) c += (uint32_t)popc_row(m[d]);
    cnt[k] = c;
    any[k] = VCap > 0 ? (m[0] | m[1] | m[2] | m[3] | m[4] | m[5]) : (RowT)0;
    local += c;
    if (VCap > 0) vl += (uint32_t)popc_row(any[k]);
    nzl += c != 0u ? 1u : 0u;
  }
  // Deterministic block scan of (faces << 40 | face voxels << 20 | rows with faces); each
  // field stays below 2^20 (at most 3N^3 + 6N^2 faces): warp inclusive scan, then a scan
  // of the warp totals.
  const int lane = t & 31, warp = t >> 5, nwarps = T >> 5;
  const unsigned long long mine =
      ((unsigned long long)local << 40) | ((unsigned long long)vl << 20) | nzl;
  unsigned long long incl = mine;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned long long v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  unsigned long long* wsum = reinterpret_cast<unsigned long long*>(s.stage);  // staging is free
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  // every warp scans the warp totals itself (no second barrier)
  unsigned long long before = 0, tot = 0;
  {
    const unsigned long long v = lane < nwarps ? wsum[lane] : 0ull;
    unsigned long long vi = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned long long u = __shfl_up_sync(0xffffffffu, vi, off);
      if (lane >= off) vi += u;
    }
    before = __shfl_sync(0xffffffffu, vi - v, warp);  // exclusive offset of this warp
    tot = __shfl_sync(0xffffffffu, vi, nwarps - 1);   // chunk totals
  }
  const unsigned long long excl = before + incl - mine;
  const uint32_t nvox = (uint32_t)(tot >> 20) & 0xFFFFFu;
  const bool use_list = VCap > 0 && nvox <= (uint32_t)VCap;
  uint32_t run = (uint32_t)(excl >> 40);
  uint32_t vrun = (uint32_t)(excl >> 20) & 0xFFFFFu;
  uint32_t nzrun = (uint32_t)excl & 0xFFFFFu;
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = t * RPT + k;
    s.rows[r] = run;
    if (cnt[k] != 0u) s.nz[nzrun++] = (uint16_t)r;
    if (VCap > 0 && use_list) {
      RowT u = any[k];
      while (u) {
        const int x = __ffs((uint32_t)u) - 1;
        u &= u - (RowT)1;
        s.vlist[vrun++] = (uint16_t)((r << Shape<N>::LOG2N) | x);
      }
    }
    run += cnt[k];
  }
  const uint32_t total = (uint32_t)(tot >> 40);
  if (t == 0) {
    s.rows[Shape<N>::R] = total;
    s.misc[0] = (int)(tot & 0xFFFFFu);
    s.misc[1] = use_list ? (int)nvox : -1;
  }
  __syncthreads();
  return total;
}

// Decoupled look-back over chunks (warp 0 of the CTA). Returns the exclusive prefix of
// chunk i. Each poll reads a window of 128 predecessors (4 per lane, coalesced), walks
// back to the nearest inclusive prefix and sums the aggregates in between. Every wait is
// bounded (spin_limit polls); on timeout the error bit is set and 0 is used.
constexpr int kLookbackWindow = 128;
// publish_agg = false: chunk i's aggregate is already published (overlap schedule).
static __device__ unsigned long long lookback(unsigned long long* state, BatchCtl* ctl,
                                              unsigned epoch, int i, unsigned long long total,
                                              int spin_limit, bool publish_agg = true) {
  const int lane = threadIdx.x & 31;
  unsigned long long excl = 0;
  if (i == 0) {
    if (lane == 0) st_relaxed_u64(&state[0], pack_state(epoch, kFlagIncl, total));
    return 0;
  }
  if (lane == 0 && publish_agg) st_relaxed_u64(&state[i], pack_state(epoch, kFlagAgg, total));
  const unsigned tag = epoch & 0xFFFFFFu;
  const unsigned long long vmask = (1ull << 38) - 1;
  int j = i - 1;
  int spins = 0;
  while (true) {
    // window position p = 32k + lane <-> chunk j - p (p = 0 is the nearest predecessor)
    unsigned long long sv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int idx = j - (32 * k + lane);
      sv[k] = idx >= 0 ? ld_relaxed_u64(&state[idx]) : pack_state(epoch, kFlagIncl, 0);
    }
    int first_incl = kLookbackWindow;
    unsigned bad[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const unsigned e = (unsigned)(sv[k] >> 40) & 0xFFFFFFu;
      const unsigned long long flag = (sv[k] >> 38) & 3ull;
      const bool valid = e == tag && flag != 0ull;
      const unsigned incl = __ballot_sync(0xffffffffu, valid && flag == kFlagIncl);
      bad[k] = __ballot_sync(0xffffffffu, !valid);
      if (first_incl == kLookbackWindow && incl) first_incl = 32 * k + __ffs(incl) - 1;
    }
    // every position up to and including first_incl must be published
    bool wait = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int hi = first_incl - 32 * k;  // positions 0..hi of this row are needed
      if (hi < 0) continue;
      const unsigned need = hi >= 31 ? 0xffffffffu : ((2u << hi) - 1u);
      if (bad[k] & need) wait = true;
    }
    if (wait) {
      if (++spins > spin_limit) {
        if (lane == 0) atomicOr(&ctl->err, ERR_TIMEOUT);
        break;
      }
      __nanosleep(spins < 8 ? 20 : 200);
      continue;
    }
    unsigned long long v = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (32 * k + lane <= first_incl) v += sv[k] & vmask;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    excl += v;
    if (first_incl < kLookbackWindow) break;
    j -= kLookbackWindow;
  }
  if (lane == 0) st_relaxed_u64(&state[i], pack_state(epoch, kFlagIncl, excl + total));
  return excl;
}

// Pulls the launch's per-chunk inputs (coordinates, neighbour masks) into L2 at the start,
// one 128-byte line per CTA and step of the grid, so that the chunks' first reads find them
// there instead of in DRAM.
__device__ __forceinline__ void prefetch_inputs(const MeshArgs& a) {
  const unsigned long long cbytes = 12ull * (unsigned long long)a.n;
  const unsigned long long mbytes = a.nbr_mask ? (unsigned long long)a.n : 0ull;
  const char* cp = reinterpret_cast<const char*>(a.coords);
  const char* mp = reinterpret_cast<const char*>(a.nbr_mask);
  for (unsigned long long off = 128ull * blockIdx.x; off < cbytes; off += 128ull * gridDim.x)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(cp + off));
  for (unsigned long long off = 128ull * blockIdx.x; off < mbytes; off += 128ull * gridDim.x)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(mp + off));
}

// Global face index of the launch's first face (MeshArgs::base_ptr; one thread reads it).
__device__ __forceinline__ unsigned long long launch_base(const MeshArgs& a) {
  return a.base_ptr ? *reinterpret_cast<const volatile unsigned long long*>(a.base_ptr) : 0ull;
}

// Status mirror of a launch whose caller waits for it (outputs in host memory): the last
// CTA to finish copies the error word, with kMirrorValid set, into a page-locked host word,
// so that the host reads the status after the stream sync without a device-to-host copy.
// Every earlier launch on the stream has completed, so the word holds their bits too.
__device__ __forceinline__ void finish_launch(const MeshArgs& a) {
  if (a.err_mirror == nullptr) return;
  __syncthreads();  // this CTA's error bits are set
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&a.ctl->done, 1u) == gridDim.x - 1u) {
      __threadfence();
      const unsigned e = atomicOr(&a.ctl->err, 0u);
      a.ctl->done = 0u;
      *reinterpret_cast<volatile unsigned*>(a.err_mirror) = e | kMirrorValid;
    }
  }
}

// Staging-buffer placement of window records. The index records (vertex layout) and the
// instance records are shifted so that the bulk-copied part starts on a 16-byte boundary
// in shared and in global memory (global face g0 + l0 with (g0 + l0) even, resp. a
// multiple of 4).
template <int LAYOUT>
__device__ __forceinline__ int stage_shift(unsigned long long g) {
  if (LAYOUT == VOX_LAYOUT_INSTANCED) {
    const int l0 = (int)((4u - (unsigned)(g & 3ull)) & 3u);
    return (16 - 4 * l0) & 15;
  }
  return (g & 1ull) ? 8 : 0;
}

// Writes face l of the staging window (chunk-local index f_local) for voxel (x, y, z).
template <int LAYOUT>
__device__ __forceinline__ void stage_face(unsigned char* stage, int stage_faces, int shift, int l,
                                           int dir, float tx, float ty, float tz, uint32_t f_local,
                                           const TablesDev* tab) {
  if (LAYOUT == VOX_LAYOUT_INSTANCED) {
    uint32_t* o = reinterpret_cast<uint32_t*>(stage + shift + (size_t)l * 68);
    const float z0 = tx * 0.0f, z1 = ty * 0.0f, z2 = tz * 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      o[4 * c + 0] = __float_as_uint(tab->part[dir][0][c] + z0);
      o[4 * c + 1] = __float_as_uint(tab->part[dir][1][c] + z1);
      o[4 * c + 2] = __float_as_uint(tab->part[dir][2][c] + z2);
      o[4 * c + 3] = __float_as_uint(tab->row3[dir][c]);
    }
    o[12] = __float_as_uint(tx);
    o[13] = __float_as_uint(ty);
    o[14] = __float_as_uint(tz);
    o[15] = __float_as_uint(1.0f);
    o[16] = tab->tex[dir];
  } else {
    float4* v = reinterpret_cast<float4*>(stage + (size_t)l * 96);
    // rotated corners of the direction, 12 floats = 3 float4 (v0xyz v1xyz v2xyz v3xyz)
    const float4* C = reinterpret_cast<const float4*>(tab->corner[dir]);
    const float4 c0 = C[0], c1 = C[1], c2 = C[2];
    const float face = __uint_as_float(tab->slot[dir]);
    // tex coords of quad::VERTICES (src/quad.rs:66-87): (0,0) (1,0) (0,1) (1,1)
    v[0] = make_float4(c0.x + tx, c0.y + ty, c0.z + tz, 0.0f);
    v[1] = make_float4(0.0f, face, c0.w + tx, c1.x + ty);
    v[2] = make_float4(c1.y + tz, 1.0f, 0.0f, face);
    v[3] = make_float4(c1.z + tx, c1.w + ty, c2.x + tz, 0.0f);
    v[4] = make_float4(1.0f, face, c2.y + tx, c2.z + ty);
    v[5] = make_float4(c2.w + tz, 1.0f, 1.0f, face);
    uint2* ix = reinterpret_cast<uint2*>(stage + (size_t)stage_faces * 96 + shift + (size_t)l * 24);
    const uint32_t b = 4u * f_local;
    ix[0] = make_uint2(b + 0u, b + 2u);
    ix[1] = make_uint2(b + 1u, b + 3u);
    ix[2] = make_uint2(b + 1u, b + 2u);
  }
}

// Sends `nw` faces staged in one warp buffer to the global output starting at face
// index g: lane 0 issues the TMA bulk copies of the 16-byte aligned part and commits them
// as one bulk group; the few unaligned head/tail records are stored word by word by the
// other lanes. Call after fence.proxy.async + __syncwarp.
template <int LAYOUT>
__device__ __forceinline__ void flush_warp(const unsigned char* buf, int shift, int nw,
                                           unsigned long long g, void* out0, void* out1) {
  const int lane = threadIdx.x & 31;
  unsigned char* o0 = reinterpret_cast<unsigned char*>(out0);
  if (LAYOUT == VOX_LAYOUT_INSTANCED) {
    int l0 = (int)((4u - (unsigned)(g & 3ull)) & 3u);
    if (l0 > nw) l0 = nw;
    const int l1 = l0 + ((nw - l0) & ~3);
    const unsigned char* src = buf + shift;
    if (lane == 0) {
      if (l1 > l0)
        bulk_s2g(o0 + (g + l0) * 68ull, src + (size_t)l0 * 68, (uint32_t)(l1 - l0) * 68u);
      bulk_commit();
    }
    // head faces [0, l0) and tail faces [l1, nw), 17 words each
    const int head = l0 * 17, tail = (nw - l1) * 17;
    for (int q = lane - 1; q >= 0 && q < head + tail; q += 31) {
      const int w = q < head ? q : (l1 * 17 + (q - head));
      reinterpret_cast<uint32_t*>(o0 + g * 68ull)[w] = reinterpret_cast<const uint32_t*>(src)[w];
    }
  } else {
    unsigned char* o1 = reinterpret_cast<unsigned char*>(out1);
    const int l0 = (int)(g & 1ull) < nw ? (int)(g & 1ull) : nw;
    const int l1 = l0 + ((nw - l0) & ~1);
    const unsigned char* isrc = buf + kWarpBatch * 96 + shift;
    if (lane == 0) {
      bulk_s2g(o0 + g * 96ull, buf, (uint32_t)nw * 96u);
      if (l1 > l0)
        bulk_s2g(o1 + (g + l0) * 24ull, isrc + (size_t)l0 * 24, (uint32_t)(l1 - l0) * 24u);
      bulk_commit();
    }
    const int head = l0 * 6, tail = (nw - l1) * 6;
    for (int q = lane - 1; q >= 0 && q < head + tail; q += 31) {
      const int w = q < head ? q : (l1 * 6 + (q - head));
      reinterpret_cast<uint32_t*>(o1 + g * 24ull)[w] = reinterpret_cast<const uint32_t*>(isrc)[w];
    }
  }
}

// flush_warp with plain stores instead of bulk copies: the lanes copy the 16-byte aligned
// part in 16-byte units (each warp store writes 512 contiguous bytes), then the head/tail
// words. For outputs in host memory, where full-line writes matter most.
template <int LAYOUT>
__device__ __forceinline__ void flush_warp_lanes(const unsigned char* buf, int shift, int nw,
                                                 unsigned long long g, void* out0, void* out1) {
  const int lane = threadIdx.x & 31;
  unsigned char* o0 = reinterpret_cast<unsigned char*>(out0);
  if (LAYOUT == VOX_LAYOUT_INSTANCED) {
    int l0 = (int)((4u - (unsigned)(g & 3ull)) & 3u);
    if (l0 > nw) l0 = nw;
    const int l1 = l0 + ((nw - l0) & ~3);
    const unsigned char* src = buf + shift;
    const uint4* s16 = reinterpret_cast<const uint4*>(src + (size_t)l0 * 68);
    uint4* d16 = reinterpret_cast<uint4*>(o0 + (g + l0) * 68ull);
    for (int q = lane; q < (l1 - l0) * 68 / 16; q += 32) d16[q] = s16[q];
    const int head = l0 * 17, tail = (nw - l1) * 17;
    for (int q = lane; q < head + tail; q += 32) {
      const int w = q < head ? q : (l1 * 17 + (q - head));
      reinterpret_cast<uint32_t*>(o0 + g * 68ull)[w] = reinterpret_cast<const uint32_t*>(src)[w];
    }
  } else {
    unsigned char* o1 = reinterpret_cast<unsigned char*>(out1);
    const int l0 = (int)(g & 1ull) < nw ? (int)(g & 1ull) : nw;
    const int l1 = l0 + ((nw - l0) & ~1);
    const unsigned char* isrc = buf + kWarpBatch * 96 + shift;
    const uint4* v16 = reinterpret_cast<const uint4*>(buf);
    uint4* dv = reinterpret_cast<uint4*>(o0 + g * 96ull);
    for (int q = lane; q < nw * 6; q += 32) dv[q] = v16[q];
    const uint4* i16 = reinterpret_cast<const uint4*>(isrc + (size_t)l0 * 24);
    uint4* di = reinterpret_cast<uint4*>(o1 + (g + l0) * 24ull);
    for (int q = lane; q < (l1 - l0) * 24 / 16; q += 32) di[q] = i16[q];
    const int head = l0 * 6, tail = (nw - l1) * 6;
    for (int q = lane; q < head + tail; q += 32) {
      const int w = q < head ? q : (l1 * 6 + (q - head));
      reinterpret_cast<uint32_t*>(o1 + g * 24ull)[w] = reinterpret_cast<const uint32_t*>(isrc)[w];
    }
  }
}

// A face of a warp's face list: local voxel (x, y, z) and emission direction.
__device__ __forceinline__ uint32_t pack_face(int x, int y, int z, int d) {
  return (uint32_t)x | ((uint32_t)y << 7) | ((uint32_t)z << 14) | ((uint32_t)d << 21);
}

// Face compaction of one warp: lane l owns element base + l of the chunk's emission
// elements, the face voxels of s.vlist (use_list) or else every voxel of the rows with
// faces (rows nz[], N voxels each); either way the warp's voxels are consecutive in
// emission order. Each lane lists its voxel's faces in direction order into the warp's
// face list; returns the warp's face count and, in `first`, the chunk-relative index of
// the warp's first face (face i of the list has index first + i).
template <int N, int LAYOUT>
__device__ __forceinline__ int warp_faces(const ChunkSmem<N, LAYOUT>& s, bool use_list,
                                          int elems, int base, uint32_t* list, uint32_t& first) {
  using RowT = typename Shape<N>::RowT;
  const int lane = threadIdx.x & 31;
  const int e = base + lane;
  unsigned bits = 0;
  uint32_t mine = 0;
  int x = 0, y = 0, z = 0;
  if (e < elems) {
    int r;
    if (Shape<N>::VCap > 0 && use_list) {
      const uint32_t q = s.vlist[e];
      x = (int)(q & (uint32_t)(N - 1));
      r = (int)(q >> Shape<N>::LOG2N);
    } else {
      r = s.nz[e / N];
      x = e % N;
    }
    y = r / N;
    z = r % N;
    RowT m[6];
    row_masks<N, LAYOUT>(s, y, z, m);
#pragma unroll
    for (int d = 0; d < 6; ++d) bits |= (unsigned)((m[d] >> x) & (RowT)1) << d;
    // Only lane 0's position is needed (the warp scan places the others): the row's face
    // offset plus the faces of the voxels before x in the row.
    uint32_t pre = 0;
    if (lane == 0 && x != 0) {
      const RowT below = (RowT)(~(RowT)0) >> (sizeof(RowT) * 8 - x);
#pragma unroll
      for (int d = 0; d < 6; ++d) pre += (uint32_t)popc_row(m[d] & below);
    }
    mine = s.rows[r] + pre;
  }
  const int cnt = __popc(bits);
  int incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  first = __shfl_sync(0xffffffffu, mine, 0);  // lane 0's voxel starts the warp's range
  int pos = incl - cnt;
  while (bits) {
    const int d = __ffs(bits) - 1;
    bits &= bits - 1u;
    list[pos++] = pack_face(x, y, z, d);
  }
  __syncwarp();
  return total;
}

// Emission elements of the chunk in shared memory: listed face voxels, or every voxel of
// the rows with faces.
template <int N, int LAYOUT>
__device__ __forceinline__ int emit_elems(const ChunkSmem<N, LAYOUT>& s) {
  return s.misc[1] >= 0 ? s.misc[1] : s.misc[0] * N;
}

// Emits the faces of the chunk in reference order: chunk-local face f goes to global
// face g0 + f. Every warp compacts the faces of its 32 voxels, stages them 32 at a time
// in one of its two shared-memory buffers (one face record per lane, final byte layout)
// and sends each batch to global memory with a TMA bulk copy issued by its lane 0. A
// warp has nbuf (1 or 2) such buffers. No CTA-wide barrier: a warp waits only until the
// bulk copy that last read a buffer is done before refilling it, and until all its
// copies have read shared memory at the end (the staging area is reused by the next
// chunk's generation).
// Faces per whole number of 128-byte output lines: 16 for the 96-byte vertex and 24-byte
// index records, 32 for the 68-byte instance records.
template <int LAYOUT>
__host__ __device__ constexpr unsigned line_faces() { return LAYOUT == VOX_LAYOUT_INSTANCED ? 32u : 16u; }

// Sends the nwf faces of a warp's face list (chunk-local indices first, first + 1, ...) to
// global faces g0 + first + ...: 32 at a time staged in one of the warp's nbuf buffers
// (`bufs`, buffer index b carried across calls) and sent by a TMA bulk copy, or by
// coalesced lane stores when lane_flush.
template <int N, int LAYOUT>
__device__ __forceinline__ void warp_send_faces(const TablesDev* tab, const uint32_t* list, int nwf,
                                                uint32_t first, vox_chunk_coord c,
                                                unsigned long long g0, unsigned long long cap,
                                                void* out0, void* out1, unsigned char* bufs,
                                                int nbuf, bool lane_flush, int& b) {
  constexpr int kBuf = warp_buf_bytes<LAYOUT>();
  const int ox = c.x * N, oy = c.y * N, oz = c.z * N;
  const int lane = threadIdx.x & 31;
  for (int r0 = 0, cnt = 0; r0 < nwf; r0 += cnt) {
    const unsigned long long g = g0 + first + (unsigned)r0;
    // a batch that starts off a line_faces boundary of the output ends on a later one, so
    // that the batches after it cover whole 128-byte lines
    cnt = kWarpBatch - (int)(g & (unsigned long long)(line_faces<LAYOUT>() - 1u));
    if (cnt > nwf - r0) cnt = nwf - r0;
    int nw = cnt;
    if (g >= cap) nw = 0;
    else if (g + (unsigned long long)cnt > cap) nw = (int)(cap - g);
    if (nw == 0) continue;
    unsigned char* buf = bufs + b * kBuf;
    // the copy issued nbuf batches ago read this buffer; wait until it is done reading
    if (lane == 0) {
      if (nbuf == 1) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
      else asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
    }
    __syncwarp();
    const int shift = stage_shift<LAYOUT>(g);
    if (lane < nw) {
      const uint32_t q = list[r0 + lane];
      const int x = q & 127, y = (q >> 7) & 127, z = (q >> 14) & 127, d = q >> 21;
      stage_face<LAYOUT>(buf, kWarpBatch, shift, lane, d, (float)(ox + x), (float)(oy + y),
                         (float)(oz + z), first + (uint32_t)(r0 + lane), tab);
    }
    if (lane_flush) {
      __syncwarp();
      flush_warp_lanes<LAYOUT>(buf, shift, nw, g, out0, out1);
    } else {
      fence_proxy_async_smem();
      __syncwarp();
      flush_warp<LAYOUT>(buf, shift, nw, g, out0, out1);
    }
    __syncwarp();
    b = nbuf == 2 ? b ^ 1 : 0;
  }
}

// Emission of elements [lo, hi): warp w takes the contiguous run [lo + w*per, ...) of
// whole groups of 32 elements, so consecutive groups' faces are adjacent in the output.
// Faces accumulate in the warp's list and leave once there are at least 32, up to the last
// line_faces boundary of the output (g0: the output index of chunk-local face 0); fewer
// than line_faces are carried to the next group, and the rest leave at the end. Batches
// that start and end on those boundaries write whole 128-byte lines, which matters most
// for outputs in host memory, where a partial line costs a slower write.
template <int N, int LAYOUT, typename Send>
__device__ __forceinline__ void emit_runs(ChunkSmem<N, LAYOUT>& s, int lo, int hi,
                                          unsigned long long g0, Send send) {
  constexpr unsigned kLine = line_faces<LAYOUT>();
  const unsigned phase = (unsigned)(g0 & (unsigned long long)(kLine - 1u));
  const bool use_list = s.misc[1] >= 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t* list = s.lists + warp * kWarpFaces;
  const int groups = (hi - lo + 31) >> 5;
  const int gper = (groups + nwarps - 1) / nwarps;
  const int wlo = lo + warp * gper * 32;
  const int whi = min(hi, wlo + gper * 32);
  int have = 0;             // faces waiting in list[0, have)
  uint32_t first_have = 0;  // chunk-local index of list[0]
  for (int base = wlo; base < whi; base += 32) {
    uint32_t first;
    const int nwf = warp_faces<N, LAYOUT>(s, use_list, whi, base, list + have, first);
    if (have == 0) first_have = first;
    have += nwf;
    const int full = have >= 32 ? have - (int)((phase + first_have + (unsigned)have) & (kLine - 1u)) : 0;
    if (full > 0) {
      send(list, full, first_have);
      // move the remainder (< 32 faces) to the front of the list
      const uint32_t keep = lane < have - full ? list[full + lane] : 0u;
      __syncwarp();
      if (lane < have - full) list[lane] = keep;
      __syncwarp();
      first_have += (uint32_t)full;
      have -= full;
    }
  }
  if (have > 0) send(list, have, first_have);
}

// wait_read = false: the caller's next use of the staging area is another emit_chunk. With
// one buffer per warp its first send waits for every earlier copy's read of that buffer,
// so the warp need not wait for its last copies here (with two buffers it still does: the
// next call starts again at buffer 0, which the last copy may still be reading).
template <int N, int LAYOUT>
__device__ void emit_chunk(ChunkSmem<N, LAYOUT>& s, vox_chunk_coord c, unsigned long long g0,
                           unsigned long long cap, void* out0, void* out1, int nbuf,
                           bool lane_flush, int lo, int hi, bool wait_read = true) {
  constexpr int kBuf = warp_buf_bytes<LAYOUT>();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* bufs = s.stage + (size_t)warp * nbuf * kBuf;
  int b = 0;
  emit_runs<N, LAYOUT>(s, lo, hi, g0, [&](const uint32_t* list, int nf, uint32_t first) {
    warp_send_faces<N, LAYOUT>(s.tab, list, nf, first, c, g0, cap, out0, out1, bufs, nbuf,
                               lane_flush, b);
  });
  if (wait_read || nbuf != 1) {
    if (lane == 0) bulk_wait_read_all();
    __syncwarp();
  }
}

// Writes one face record straight to global memory (face index g).
template <int LAYOUT>
__device__ __forceinline__ void store_face(void* out0, void* out1, unsigned long long g, int dir,
                                           float tx, float ty, float tz, uint32_t f_local,
                                           const TablesDev* tab) {
  if (LAYOUT == VOX_LAYOUT_INSTANCED) {
    uint32_t* o = reinterpret_cast<uint32_t*>(out0) + g * 17ull;
    const float z0 = tx * 0.0f, z1 = ty * 0.0f, z2 = tz * 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      o[4 * c + 0] = __float_as_uint(tab->part[dir][0][c] + z0);
      o[4 * c + 1] = __float_as_uint(tab->part[dir][1][c] + z1);
      o[4 * c + 2] = __float_as_uint(tab->part[dir][2][c] + z2);
      o[4 * c + 3] = __float_as_uint(tab->row3[dir][c]);
    }
    o[12] = __float_as_uint(tx);
    o[13] = __float_as_uint(ty);
    o[14] = __float_as_uint(tz);
    o[15] = __float_as_uint(1.0f);
    o[16] = tab->tex[dir];
  } else {
    float4* v = reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(out0) + g * 96ull);
    const float4* C = reinterpret_cast<const float4*>(tab->corner[dir]);
    const float4 c0 = C[0], c1 = C[1], c2 = C[2];
    const float face = __uint_as_float(tab->slot[dir]);
    v[0] = make_float4(c0.x + tx, c0.y + ty, c0.z + tz, 0.0f);
    v[1] = make_float4(0.0f, face, c0.w + tx, c1.x + ty);
    v[2] = make_float4(c1.y + tz, 1.0f, 0.0f, face);
    v[3] = make_float4(c1.z + tx, c1.w + ty, c2.x + tz, 0.0f);
    v[4] = make_float4(1.0f, face, c2.y + tx, c2.z + ty);
    v[5] = make_float4(c2.w + tz, 1.0f, 1.0f, face);
    uint2* ix = reinterpret_cast<uint2*>(reinterpret_cast<unsigned char*>(out1) + g * 24ull);
    const uint32_t b = 4u * f_local;
    ix[0] = make_uint2(b + 0u, b + 2u);
    ix[1] = make_uint2(b + 1u, b + 3u);
    ix[2] = make_uint2(b + 1u, b + 2u);
  }
}

// The direct counterpart of warp_send_faces: lane l stores faces l, l + 32, ... of the
// list straight to global memory.
template <int N, int LAYOUT>
__device__ __forceinline__ void warp_store_faces(const TablesDev* tab, const uint32_t* list, int nwf,
                                                 uint32_t first, vox_chunk_coord c,
                                                 unsigned long long g0, unsigned long long cap,
                                                 void* out0, void* out1) {
  const int ox = c.x * N, oy = c.y * N, oz = c.z * N;
  for (int i = threadIdx.x & 31; i < nwf; i += 32) {
    const uint32_t q = list[i];
    const int x = q & 127, y = (q >> 7) & 127, z = (q >> 14) & 127, d = q >> 21;
    const uint32_t l = first + (uint32_t)i;
    const unsigned long long gg = g0 + l;
    if (gg < cap)
      store_face<LAYOUT>(out0, out1, gg, d, (float)(ox + x), (float)(oy + y), (float)(oz + z),
                         l, tab);
  }
  __syncwarp();
}

// Direct variant of emit_chunk: the same runs and compaction, then every lane writes one
// face record straight to global memory (32 consecutive faces per warp step).
template <int N, int LAYOUT>
__device__ void emit_chunk_direct(ChunkSmem<N, LAYOUT>& s, vox_chunk_coord c,
                                  unsigned long long g0, unsigned long long cap, void* out0,
                                  void* out1, int lo, int hi) {
  emit_runs<N, LAYOUT>(s, lo, hi, g0, [&](const uint32_t* list, int nf, uint32_t first) {
    warp_store_faces<N, LAYOUT>(s.tab, list, nf, first, c, g0, cap, out0, out1);
  });
}

// ------------------------------------------------------------------------------------
// Kernels
// ------------------------------------------------------------------------------------

// Minimum resident CTAs per SM the fused kernels are compiled for, i.e. their register
// budget: 64 registers a thread in general (4 CTAs of 256 threads), which keeps the
// meshing paths at the occupancy their shared memory allows. The 3-D density generator
// needs more: 80 at 256 threads for 32^3 chunks (3 CTAs), 64 at 512 (2 CTAs); 16^3 and 8^3
// chunks keep the budgets the compiler chose for them unconstrained, and 64^3 density or
// heightmap chunks at 512 threads keep up to 128.
template <int N, int GM, int T>
__host__ __device__ constexpr int fused_min_ctas() {
  if (GM == GM_DENSITY) {
    if (N == 32) return T == 256 ? 3 : 2;
    if (N == 16) return T == 256 ? 3 : 7;
    if (N == 8) return T == 64 ? 14 : 25;
    return 1;
  }
  if (GM == GM_HEIGHT && N == 64 && T == 512) return 1;
  return 65536 / (T * 64) > 0 ? 65536 / (T * 64) : 1;
}

// Persistent fused generation + meshing over a device work queue (GM != GM_OCC), or
// meshing of resident occupancy (GM == GM_OCC). One chunk per CTA iteration; T threads.
// Occupancy and halo rows of chunk i in shared memory: loaded from the slot pool
// (GM_OCC) or generated from the noise field.
template <int N, int GM, int LAYOUT, int T>
__device__ __forceinline__ void prepare_chunk(ChunkSmem<N, LAYOUT>& s, const MeshArgs& a, int i,
                                              vox_chunk_coord c) {
  if (GM == GM_OCC) {
    const unsigned long long words = (unsigned long long)N * N * Shape<N>::W;
    const int slot = a.slots[i];
    const uint32_t* nb[6];
    unsigned use = 0;
    bool bad = slot < 0 || slot >= a.pool_slots;
    for (int d = 0; d < 6; ++d) {
      const int ns = a.nbr_slots ? a.nbr_slots[6 * i + d] : -1;
      nb[d] = nullptr;
      if (d >= 4 && !a.full6) continue;
      if (ns >= a.pool_slots) bad = true;
      if (ns >= 0 && ns < a.pool_slots) {
        nb[d] = a.occ_pool + (unsigned long long)ns * words;
        use |= 1u << d;
      }
    }
    if (bad && threadIdx.x == 0) atomicOr(&a.ctl->err, ERR_BAD_INPUT);
    // An out-of-range slot reads slot 0 instead (the call then reports VOX_ERR_INVALID).
    const int sl = (slot >= 0 && slot < a.pool_slots) ? slot : 0;
    load_chunk<N, LAYOUT>(s, a.occ_pool + (unsigned long long)sl * words, nb, use);
  } else {
    unsigned m = a.nbr_mask ? a.nbr_mask[i] : 0u;
    if (GM == GM_BERNOULLI) m = 0u;
    if (!a.full6) m &= 0xFu;
    gen_chunk<N, GM, LAYOUT, T>(s, a.gen, c, a.index_base + i, m, true);
  }
}

template <int N, int GM, int LAYOUT, int T>
__global__ void __launch_bounds__(T, fused_min_ctas<N, GM, T>())
k_mesh_batch(const __grid_constant__ MeshArgs a, const __grid_constant__ TablesDev tab) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, LAYOUT> s;
  s.carve(smem_raw);
  load_tables<N, LAYOUT>(s, &tab);  // the tables travel as a kernel parameter
  __shared__ int s_item;
  __shared__ unsigned long long s_base, s_base0;
  __shared__ unsigned s_epoch;
  if (threadIdx.x == 0) {
    s_epoch = ld_relaxed_u32(&a.ctl->epoch);
    s_base0 = launch_base(a);
    __threadfence();
    s_item = (int)atomicAdd(&a.ctl->next, 1u);
  }
  __syncthreads();
  const unsigned epoch = s_epoch;
  const unsigned long long base0 = s_base0;
  int i = s_item;
  while (true) {
    if (i >= a.n) {
      if (threadIdx.x == 0 && i == a.n + (int)gridDim.x - 1) {
        // The last ticket of this launch: reset the queue and advance the epoch.
        a.ctl->next = 0u;
        a.ctl->epoch = epoch + 1u;
      }
      break;
    }
    // The next ticket is drawn now and used after this chunk, so the atomic's latency
    // overlaps the chunk's work. A CTA reserves chunks in increasing order, so the
    // lowest unfinished chunk is always being processed and every look-back ends.
    int next_item = 0;
    if (threadIdx.x == 0) next_item = (int)atomicAdd(&a.ctl->next, 1u);
    const vox_chunk_coord c = a.coords[i];
    prepare_chunk<N, GM, LAYOUT, T>(s, a, i, c);
    const uint32_t total = count_and_scan<N, LAYOUT, T>(s);
    if (threadIdx.x < 32) {
      const unsigned long long excl =
          base0 + lookback(a.state, a.ctl, epoch, i, total, a.spin_limit);
      if (threadIdx.x == 0) {
        s_base = excl;
        a.face_offsets[i] = excl;
        if (i == a.n - 1) {
          a.face_offsets[a.n] = excl + total;
          if (excl + total > a.cap) atomicOr(&a.ctl->err, ERR_CAPACITY);
        }
      }
    }
    __syncthreads();
    if (a.stage_faces > 0)
      emit_chunk<N, LAYOUT>(s, c, s_base, a.cap, a.out0, a.out1, a.stage_faces / kWarpBatch,
                            a.lane_flush != 0, 0, emit_elems(s));
    else emit_chunk_direct<N, LAYOUT>(s, c, s_base, a.cap, a.out0, a.out1, 0, emit_elems(s));
    if (threadIdx.x == 0) s_item = next_item;
    __syncthreads();
    i = s_item;
  }
  if ((threadIdx.x & 31) == 0) bulk_wait_all();  // every lane 0 issued bulk copies
  finish_launch(a);
}

// ------------------------------------------------------------------------------------
// Phased schedule of the fused batch kernel (cooperative launch: the whole grid is
// resident, so CTAs may wait for one another).
//  A. CTAs take chunks from the work queue, prepare and count them, and spill the chunk
//     state (occupancy, halo, row offsets, row and voxel lists) to a per-chunk slot
//     (L2-resident) and the face total to counts[i].
//  B. Grid barrier (it also resets the queue). CTA 0 scans counts[] into face_offsets[]
//     and raises the scan flag.
//  C. CTAs take emission items (a chunk, or a segment of one) from the queue again,
//     reload the chunk state, wait for the scan flag once, and emit at face_offsets[i].
// There is no chunk-to-chunk dependency inside a phase. The output bytes are the same
// as the look-back schedule's.
// ------------------------------------------------------------------------------------

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier, called by thread 0 of every CTA after a __syncthreads. The last CTA to
// arrive resets the arrival count and the first work queue, then advances the
// generation; the others poll the generation at most spin_limit times. Returns the new
// generation, or 0xFFFFFFFF after a timeout (ERR_TIMEOUT is set).
static __device__ unsigned grid_barrier_t0(BatchCtl* ctl, unsigned nblocks, int spin_limit) {
  const unsigned gen = ld_acquire_u32(&ctl->bar_gen);
  __threadfence();  // this CTA's earlier writes are visible before its arrival
  const unsigned arrived = atomicAdd(&ctl->bar_count, 1u);
  if (arrived == nblocks - 1u) {
    ctl->bar_count = 0u;
    ctl->next = 0u;
    __threadfence();
    st_release_u32(&ctl->bar_gen, gen + 1u);
    return gen + 1u;
  }
  int spins = 0;
  while (ld_acquire_u32(&ctl->bar_gen) == gen) {
    if (++spins > spin_limit) {
      atomicOr(&ctl->err, ERR_TIMEOUT);
      return 0xFFFFFFFFu;
    }
    __nanosleep(spins < 8 ? 32 : 256);
  }
  __threadfence();
  return gen + 1u;
}

// Deterministic exclusive scan of counts[0, n) into offs[0, n) starting at `base`, base +
// total at offs[n] (one CTA of T threads, 8 counts per thread per tile). Returns base + total.
template <int T>
__device__ unsigned long long scan_counts(const uint32_t* counts, int n,
                                          unsigned long long* offs, unsigned long long* wsum,
                                          unsigned long long base) {
  constexpr int V = 8;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarps = T >> 5;
  unsigned long long carry = base;
  for (int base = 0; base < n; base += T * V) {
    uint32_t v[V];
    unsigned long long local = 0;
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const int idx = base + t * V + k;
      v[k] = idx < n ? __ldcg(counts + idx) : 0u;
      local += v[k];
    }
    unsigned long long incl = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned long long u = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += u;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const unsigned long long w = lane < nwarps ? wsum[lane] : 0ull;
      unsigned long long wi = w;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long u = __shfl_up_sync(0xffffffffu, wi, off);
        if (lane >= off) wi += u;
      }
      if (lane < nwarps) wsum[32 + lane] = wi - w;
      if (lane == nwarps - 1) wsum[64] = wi;
    }
    __syncthreads();
    unsigned long long run = carry + wsum[32 + warp] + incl - local;
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const int idx = base + t * V + k;
      if (idx < n) offs[idx] = run;
      run += v[k];
    }
    carry += wsum[64];
    __syncthreads();  // wsum is reused by the next tile
  }
  if (t == 0) offs[n] = carry;
  return carry;
}

template <int N, int GM, int LAYOUT, int T>
__global__ void __launch_bounds__(T, fused_min_ctas<N, GM, T>())
k_mesh_batch_phased(const __grid_constant__ MeshArgs a, const __grid_constant__ TablesDev tab) {
  using P = SmemPlan<N, LAYOUT>;
  // spill slot of a chunk: [occ | halo | rows] [nz] [vlist] [misc], laid out as in shared
  // memory; the lists are copied only as far as they are used
  constexpr int kFixed16 = (P::kOcc + P::kHalo + P::kRows) / 16;
  constexpr int kNzOff = P::kOcc + P::kHalo + P::kRows;
  constexpr int kVlOff = kNzOff + P::kNz;
  constexpr int kMiscOff = kVlOff + P::kVList;
  static_assert(P::kSpill == kMiscOff + P::kMisc, "spill layout");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, LAYOUT> s;
  s.carve(smem_raw);
  load_tables<N, LAYOUT>(s, &tab);  // the tables travel as a kernel parameter
  __shared__ int s_item;
  __shared__ unsigned s_gen;
  __shared__ unsigned long long s_base;
  unsigned char* const spill = reinterpret_cast<unsigned char*>(a.scratch);
  uint4* const fixed16 = reinterpret_cast<uint4*>(s.occ);  // s.halo, s.rows follow s.occ
  const int t = threadIdx.x;
  __syncthreads();

  // A. prepare + count + spill (the next ticket is drawn before the chunk's work)
  if (t == 0) s_item = (int)atomicAdd(&a.ctl->next, 1u);
  __syncthreads();
  for (int i = s_item; i < a.n;) {
    int next_item = 0;
    if (t == 0) next_item = (int)atomicAdd(&a.ctl->next, 1u);
    prepare_chunk<N, GM, LAYOUT, T>(s, a, i, a.coords[i]);
    const uint32_t total = count_and_scan<N, LAYOUT, T>(s);
    unsigned char* dst = spill + (unsigned long long)i * P::kSpill;
    for (int q = t; q < kFixed16; q += T) __stcg(reinterpret_cast<uint4*>(dst) + q, fixed16[q]);
    const int nzw = (s.misc[0] + 1) >> 1;                          // u32 words of nz used
    const int vlw = s.misc[1] > 0 ? (s.misc[1] + 1) >> 1 : 0;      // u32 words of vlist used
    for (int q = t; q < nzw; q += T)
      __stcg(reinterpret_cast<uint32_t*>(dst + kNzOff) + q, reinterpret_cast<const uint32_t*>(s.nz)[q]);
    for (int q = t; q < vlw; q += T)
      __stcg(reinterpret_cast<uint32_t*>(dst + kVlOff) + q,
             reinterpret_cast<const uint32_t*>(s.vlist)[q]);
    if (t == 0) {
      __stcg(reinterpret_cast<int2*>(dst + kMiscOff), make_int2(s.misc[0], s.misc[1]));
      __stcg(a.counts + i, total);
      s_item = next_item;
    }
    __syncthreads();
    i = s_item;
  }

  // B. barrier; CTA 0 scans the counts
  __syncthreads();
  if (t == 0) s_gen = grid_barrier_t0(a.ctl, gridDim.x, a.spin_limit);
  __syncthreads();
  const unsigned gen = s_gen;
  if (gen == 0xFFFFFFFFu) return;
  if (blockIdx.x == 0) {
    if (t == 0) s_base = launch_base(a);
    __syncthreads();
    const unsigned long long total = scan_counts<T>(a.counts, a.n, a.face_offsets,
                                                    reinterpret_cast<unsigned long long*>(s.stage),
                                                    s_base);
    __syncthreads();
    if (t == 0) {
      if (total > a.cap) atomicOr(&a.ctl->err, ERR_CAPACITY);
      __threadfence();
      st_release_u32(&a.ctl->scan_flag, gen);
    }
  }

  // C. emission items from the work queue: item k is segment k % split of chunk
  // k / split (the chunk's emission elements cut into split runs of whole warp batches).
  // The chunk state comes back from the spill slot, so nothing is counted twice.
  const int split = a.split > 0 ? a.split : 1;
  const int items = a.n * split;
  bool scanned = blockIdx.x == 0;  // thread 0's view: the scan flag has been seen
  if (t == 0) s_item = (int)atomicAdd(&a.ctl->next, 1u);
  __syncthreads();
  int k = s_item;
  while (true) {
    if (k >= items) {
      // The last ticket of this launch resets the queue.
      if (t == 0 && k == items + (int)gridDim.x - 1) a.ctl->next = 0u;
      break;
    }
    int next_item = 0;
    if (t == 0) next_item = (int)atomicAdd(&a.ctl->next, 1u);
    const int i = k / split, seg = k - i * split;
    const unsigned char* src = spill + (unsigned long long)i * P::kSpill;
    for (int q = t; q < kFixed16; q += T) fixed16[q] = __ldcg(reinterpret_cast<const uint4*>(src) + q);
    if (t == 0) {
      const int2 m = __ldcg(reinterpret_cast<const int2*>(src + kMiscOff));
      s.misc[0] = m.x;
      s.misc[1] = m.y;
    }
    __syncthreads();
    const bool use_list = s.misc[1] >= 0;
    const int elems = emit_elems(s);
    const int per = ((elems + split - 1) / split + 31) & ~31;
    const int lo = min(elems, seg * per), hi = min(elems, lo + per);
    if (lo < hi) {
      // the list entries that elements [lo, hi) read
      const int e0 = use_list ? lo : lo / N, e1 = use_list ? hi : (hi - 1) / N + 1;
      const uint32_t* lsrc = reinterpret_cast<const uint32_t*>(src + (use_list ? kVlOff : kNzOff));
      uint32_t* ldst = reinterpret_cast<uint32_t*>(use_list ? s.vlist : s.nz);
      for (int q = (e0 >> 1) + t; q < (e1 + 1) >> 1; q += T) ldst[q] = __ldcg(lsrc + q);
    }
    if (t == 0) {
      int spins = 0;
      while (!scanned) {
        if (ld_acquire_u32(&a.ctl->scan_flag) == gen) {
          scanned = true;
          break;
        }
        if (++spins > a.spin_limit) break;
        __nanosleep(spins < 8 ? 32 : 256);
      }
      if (scanned) {
        s_base = __ldcg(a.face_offsets + i);
      } else {
        atomicOr(&a.ctl->err, ERR_TIMEOUT);
        s_base = ~0ull;
      }
    }
    __syncthreads();
    if (s_base == ~0ull) break;  // the scan flag never came: give up (error reported)
    if (lo < hi) {
      const vox_chunk_coord c = a.coords[i];
      if (a.stage_faces > 0)
        emit_chunk<N, LAYOUT>(s, c, s_base, a.cap, a.out0, a.out1, a.stage_faces / kWarpBatch,
                              a.lane_flush != 0, lo, hi, false);
      else emit_chunk_direct<N, LAYOUT>(s, c, s_base, a.cap, a.out0, a.out1, lo, hi);
    }
    if (t == 0) s_item = next_item;
    __syncthreads();
    k = s_item;
  }
  if ((t & 31) == 0) bulk_wait_all();  // every lane 0 issued bulk copies
}

// ------------------------------------------------------------------------------------
// Overlap schedule of the fused batch kernel: the phases of k_mesh_batch_phased without
// the grid barrier, interleaved on one work queue. A generation item (A) prepares and
// counts a chunk, spills its state and publishes its face total as an epoch-tagged
// aggregate look-back state; an emission item (C) waits until its own chunk is published,
// takes the chunk's offset from a decoupled look-back over the published totals, reloads
// the chunk state and emits. Ticket order (overlap_ticket): A(0..L-1), then A(L+m) and
// C(m) alternately while generation items remain, then the remaining emission items.
// Every wait is for an item with a smaller ticket, which a running CTA holds or has
// finished, and generation items never wait, so every wait ends without co-residency:
// a normal launch. L = n (all generation first) suits launches bound by issue; a smaller L
// starts emission early, which hides generation behind a slow output (host memory).
// ------------------------------------------------------------------------------------

template <int N, int GM, int LAYOUT, int T>
__global__ void __launch_bounds__(T, fused_min_ctas<N, GM, T>())
k_mesh_batch_overlap(const __grid_constant__ MeshArgs a, const __grid_constant__ TablesDev tab) {
  using P = SmemPlan<N, LAYOUT>;
  constexpr int kFixed16 = (P::kOcc + P::kHalo + P::kRows) / 16;
  constexpr int kNzOff = P::kOcc + P::kHalo + P::kRows;
  constexpr int kVlOff = kNzOff + P::kNz;
  constexpr int kMiscOff = kVlOff + P::kVList;
  static_assert(P::kSpill == kMiscOff + P::kMisc, "spill layout");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, LAYOUT> s;
  s.carve(smem_raw);
  load_tables<N, LAYOUT>(s, &tab);  // the tables travel as a kernel parameter
  __shared__ unsigned s_item;
  __shared__ unsigned s_epoch;
  __shared__ unsigned long long s_base, s_base0;
  unsigned char* const spill = reinterpret_cast<unsigned char*>(a.scratch);
  uint4* const fixed16 = reinterpret_cast<uint4*>(s.occ);  // s.halo, s.rows follow s.occ
  const int t = threadIdx.x;
  if (t == 0) {
    prefetch_inputs(a);
    s_epoch = ld_relaxed_u32(&a.ctl->epoch);
    s_base0 = launch_base(a);
    __threadfence();
    s_item = atomicAdd(&a.ctl->next, 1u);
  }
  __syncthreads();
  const unsigned epoch = s_epoch;
  const unsigned long long base0 = s_base0;
  const unsigned tag = epoch & 0xFFFFFFu;
  const unsigned n = (unsigned)a.n;
  const int split = a.split > 0 ? a.split : 1;
  const unsigned items = n * (unsigned)split;
  const unsigned lag = a.lag < 0 || (unsigned)a.lag > n ? n : (unsigned)a.lag;
  const unsigned last_ticket = n + items + gridDim.x - 1u;
  bool stage_busy = false;  // bulk copies of this CTA may still read the staging area
  unsigned tk = s_item;
  while (true) {
    unsigned idx;
    const int kind = overlap_ticket(tk, n, items, lag, idx);
    if (kind == 2) {
      // The last ticket of this launch resets the queue and advances the epoch.
      if (t == 0 && tk == last_ticket) {
        a.ctl->next = 0u;
        a.ctl->epoch = epoch + 1u;
      }
      break;
    }
    // the next ticket is drawn now and used after this item, so the atomic's latency
    // overlaps the item's work
    unsigned next_tk = 0;
    if (t == 0) next_tk = atomicAdd(&a.ctl->next, 1u);
    if (kind == 0) {
      // A. prepare + count + spill + publish the chunk's total. Generation reuses the
      // staging area as scratch: wait until the earlier copies have read it.
      if (stage_busy) {
        if ((t & 31) == 0) bulk_wait_read_all();
        __syncthreads();
        stage_busy = false;
      }
      const int i = (int)idx;
      prepare_chunk<N, GM, LAYOUT, T>(s, a, i, a.coords[i]);
      const uint32_t total = count_and_scan<N, LAYOUT, T>(s);
      unsigned char* dst = spill + (unsigned long long)i * P::kSpill;
      // an empty chunk (no row with faces) spills only its counts: its emission item
      // reloads nothing
      if (s.misc[0] > 0)
        for (int q = t; q < kFixed16; q += T) __stcg(reinterpret_cast<uint4*>(dst) + q, fixed16[q]);
      const int nzw = (s.misc[0] + 1) >> 1;
      const int vlw = s.misc[1] > 0 ? (s.misc[1] + 1) >> 1 : 0;
      for (int q = t; q < nzw; q += T)
        __stcg(reinterpret_cast<uint32_t*>(dst + kNzOff) + q, reinterpret_cast<const uint32_t*>(s.nz)[q]);
      for (int q = t; q < vlw; q += T)
        __stcg(reinterpret_cast<uint32_t*>(dst + kVlOff) + q,
               reinterpret_cast<const uint32_t*>(s.vlist)[q]);
      __syncthreads();  // every store of the slot precedes the publication below
      if (t == 0) {
        __stcg(reinterpret_cast<int2*>(dst + kMiscOff), make_int2(s.misc[0], s.misc[1]));
        __threadfence();
        st_relaxed_u64(&a.state[i], pack_state(epoch, i == 0 ? kFlagIncl : kFlagAgg, total));
      }
    } else {
      // C. emission item idx: segment idx % split of chunk idx / split
      const int c_i = (int)(idx / (unsigned)split), seg = (int)(idx % (unsigned)split);
      const unsigned char* src = spill + (unsigned long long)c_i * P::kSpill;
      // Every thread waits for the chunk's published state with an acquire load, so its
      // own reads of the spill slot below are ordered after the slot's stores (no fence
      // and no barrier before the reload). The waits are bounded; the barrier below
      // combines them.
      unsigned long long w = 0;
      int ok = 0;
      for (int spins = 0;;) {
        w = ld_acquire_u64(&a.state[c_i]);
        if (((unsigned)(w >> 40) & 0xFFFFFFu) == tag && ((w >> 38) & 3ull) != 0ull) {
          ok = 1;
          break;
        }
        if (++spins > a.spin_limit) break;
        __nanosleep(spins < 8 ? 32 : 256);
      }
      ok = __all_sync(0xffffffffu, ok);  // warp-uniform (warp 0's look-back needs every lane)
      if (!ok && (t & 31) == 0) atomicOr(&a.ctl->err, ERR_TIMEOUT);
      // Warp 0 takes the chunk's offset by look-back over the published totals while the
      // other warps reload the chunk's state (a one-warp CTA does both, in turn).
      constexpr int TR = T > 32 ? T - 32 : 32;  // reloading threads
      const int tr = T > 32 ? t - 32 : t;
      if (t < 32 && ok) {
        // the chunk's face total (an empty chunk spilled only its counts: total 0)
        const int rows_with_faces = __ldcg(reinterpret_cast<const int*>(src + kMiscOff));
        const unsigned long long total =
            rows_with_faces > 0
                ? __ldcg(reinterpret_cast<const uint32_t*>(src + P::kOcc + P::kHalo) + Shape<N>::R)
                : 0ull;
        // An inclusive state (chunk 0, or a segment of a chunk whose offset another item
        // has already found) gives the offset at once.
        w = __shfl_sync(0xffffffffu, w, 0);
        const unsigned long long excl =
            base0 + (((w >> 38) & 3ull) == kFlagIncl
                         ? (w & ((1ull << 38) - 1)) - total
                         : lookback(a.state, a.ctl, epoch, c_i, total, a.spin_limit, false));
        if (t == 0) {
          s_base = excl;
          if (seg == 0) {
            a.face_offsets[c_i] = excl;
            if (c_i == a.n - 1) {
              a.face_offsets[a.n] = excl + total;
              if (excl + total > a.cap) atomicOr(&a.ctl->err, ERR_CAPACITY);
            }
          }
        }
      }
      if (ok && tr >= 0) {
        const int2 m = __ldcg(reinterpret_cast<const int2*>(src + kMiscOff));
        if (tr == 0) {
          s.misc[0] = m.x;
          s.misc[1] = m.y;
        }
        if (m.x > 0) {  // rows with faces: an empty chunk needs no state
          for (int q = tr; q < kFixed16; q += TR) fixed16[q] = __ldcg(reinterpret_cast<const uint4*>(src) + q);
          const bool use_list = m.y >= 0;
          const int elems = use_list ? m.y : m.x * N;
          const int per = ((elems + split - 1) / split + 31) & ~31;
          const int lo = min(elems, seg * per), hi = min(elems, lo + per);
          if (lo < hi) {
            const int e0 = use_list ? lo : lo / N, e1 = use_list ? hi : (hi - 1) / N + 1;
            const uint32_t* lsrc = reinterpret_cast<const uint32_t*>(src + (use_list ? kVlOff : kNzOff));
            uint32_t* ldst = reinterpret_cast<uint32_t*>(use_list ? s.vlist : s.nz);
            for (int q = (e0 >> 1) + tr; q < (e1 + 1) >> 1; q += TR) ldst[q] = __ldcg(lsrc + q);
          }
        }
      }
      if (!__syncthreads_and(ok)) break;  // never published (error reported)
      const int elems = emit_elems(s);
      const int per = ((elems + split - 1) / split + 31) & ~31;
      const int lo = min(elems, seg * per), hi = min(elems, lo + per);
      if (lo < hi) {
        const vox_chunk_coord c = a.coords[c_i];
        if (a.stage_faces > 0) {
          emit_chunk<N, LAYOUT>(s, c, s_base, a.cap, a.out0, a.out1, a.stage_faces / kWarpBatch,
                                a.lane_flush != 0, lo, hi, false);
          stage_busy = true;
        } else {
          emit_chunk_direct<N, LAYOUT>(s, c, s_base, a.cap, a.out0, a.out1, lo, hi);
        }
      }
    }
    if (t == 0) s_item = next_tk;
    __syncthreads();
    tk = s_item;
  }
  if ((t & 31) == 0) bulk_wait_all();  // every lane 0 issued bulk copies
  finish_launch(a);
}

// Plain per-chunk mesher: one chunk, one CTA, one launch (no queue, no look-back).
template <int N, int LAYOUT, int T>
__global__ void __launch_bounds__(T)
k_mesh_single(MeshArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, LAYOUT> s;
  s.carve(smem_raw);
  load_tables<N, LAYOUT>(s, a.tables);
  unsigned use = 0;
  for (int d = 0; d < 6; ++d)
    if (a.occ_nbr[d] && (d < 4 || a.full6)) use |= 1u << d;
  load_chunk<N, LAYOUT>(s, a.occ_self, a.occ_nbr, use);
  const uint32_t total = count_and_scan<N, LAYOUT, T>(s);
  if (threadIdx.x == 0) {
    a.face_offsets[0] = total;
    if ((unsigned long long)total > a.cap) atomicOr(&a.ctl->err, ERR_CAPACITY);
  }
  if (a.stage_faces > 0)
    emit_chunk<N, LAYOUT>(s, a.coord_single, 0ull, a.cap, a.out0, a.out1, a.stage_faces / kWarpBatch,
                          a.lane_flush != 0, 0, emit_elems(s));
  else emit_chunk_direct<N, LAYOUT>(s, a.coord_single, 0ull, a.cap, a.out0, a.out1, 0, emit_elems(s));
  if ((threadIdx.x & 31) == 0) bulk_wait_all();
}

// Register budget of k_generate as resident CTAs per SM: 64 registers a thread for the 3-D
// density noise (its lane = z loop holds a block of sums and four corner records), 32 for
// the heightmap columns up to 32^3 and for Bernoulli fills, whose occupancy then follows
// shared memory alone.
template <int N, int GM, int T>
__host__ __device__ constexpr int generate_min_ctas() {
  if (GM == GM_DENSITY || (GM == GM_HEIGHT && N > 32)) return 65536 / (T * 64) > 0 ? 65536 / (T * 64) : 1;
  return 65536 / (T * 32) > 32 ? 32 : 65536 / (T * 32);
}

// Chunk::new for n chunks, occupancy rows written to global memory. One CTA per chunk:
// chunk i at occ_out + i * words, or at slot a.slots[i] of a pool of a.pool_slots slots when
// a.slots is set (an out-of-range slot writes nothing and latches ERR_BAD_INPUT).
template <int N, int GM, int T>
__global__ void __launch_bounds__(T, generate_min_ctas<N, GM, T>())
k_generate(MeshArgs a, uint32_t* occ_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, VOX_LAYOUT_VERTEX> s;
  s.carve(smem_raw);
  constexpr int words = N * N * Shape<N>::W;
  const int i = blockIdx.x;
  long long slot = i;
  if (a.slots) {
    slot = a.slots[i];
    if (slot < 0 || slot >= a.pool_slots) {
      if (threadIdx.x == 0) atomicOr(&a.ctl->err, ERR_BAD_INPUT);
      return;  // uniform across the CTA: no barrier has been reached yet
    }
  }
  load_tables<N, VOX_LAYOUT_VERTEX>(s, a.tables);
  __syncthreads();
  gen_chunk<N, GM, VOX_LAYOUT_VERTEX, T>(s, a.gen, a.coords[i], a.index_base + i, 0u, false);
  const uint32_t* src = reinterpret_cast<const uint32_t*>(s.occ);
  uint32_t* dst = occ_out + (size_t)slot * words;
  for (int q = threadIdx.x; q < words; q += blockDim.x) dst[q] = src[q];
}

// The halo planes of chunks outside a batch (the staged-halo path of the fused batch):
// for each listed chunk i below the count *a.n_dev (at most a.n), only the plane of its
// occupancy that the meshing of its neighbour in the batch reads — x = N - 1 or x = 0 for
// dirs[i] = 0 or 1 (the chunk is the batch chunk's -x or +x neighbour), z = N - 1 or 0 for
// 2 or 3, y = N - 1 or 0 for 4 or 5 — written to occ_out + i * words, every other bit zero.
// N * N samples instead of N^3; each is the sample the fused launch generates for that halo
// plane (generation is a function of the voxel's world position). A grid of a few CTAs per
// SM strides over the list, so the launch is sized before the count is known.
template <int N, int GM, int T>
__global__ void __launch_bounds__(T, 65536 / (T * 64))
k_generate_planes(MeshArgs a, const uint8_t* __restrict__ dirs, uint32_t* occ_out) {
  static_assert(GM == GM_HEIGHT || GM == GM_DENSITY, "planes of the noise generators only");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, VOX_LAYOUT_VERTEX> s;
  s.carve(smem_raw);
  constexpr int W = Shape<N>::W;
  constexpr int words = N * N * W;
  const int count = (int)min((unsigned)a.n, *a.n_dev);
  if ((int)blockIdx.x >= count) return;  // uniform across the CTA
  load_tables<N, VOX_LAYOUT_VERTEX>(s, a.tables);
  uint32_t* occw = reinterpret_cast<uint32_t*>(s.occ);
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    for (int q = threadIdx.x; q < words; q += blockDim.x) occw[q] = 0u;
    __syncthreads();  // (the first pass: also the tables)
    const vox_chunk_coord c = a.coords[i];
    const int d = dirs[i];
    const int fix = (d & 1) ? 0 : N - 1;
    const int ox = c.x * N, oy = c.y * N, oz = c.z * N;
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
      const int p = e / N, q = e % N;
      const int x = d <= 1 ? fix : q;
      const int y = d <= 3 ? p : fix;
      const int z = d <= 1 ? q : (d <= 3 ? fix : p);
      bool solid;
      if constexpr (GM == GM_HEIGHT)
        solid = y < column_k<N, VOX_LAYOUT_VERTEX>(s, a.gen, ox, oy, oz, x, z);
      else
        solid = gen_solid<N, GM, VOX_LAYOUT_VERTEX>(s, a.gen, x, y, z, ox, oy, oz, 0ull);
      if (solid) atomicOr(&occw[(y * N + z) * W + (x >> 5)], 1u << (x & 31));
    }
    __syncthreads();
    uint32_t* dst = occ_out + (size_t)i * words;
    for (int q = threadIdx.x; q < words; q += blockDim.x) dst[q] = occw[q];
    __syncthreads();  // the next plane clears s.occ
  }
}

}  // namespace vox
