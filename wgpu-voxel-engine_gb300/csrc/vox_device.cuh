// vox_device.cuh — device code of the chunk generation + meshing path (sm_103a).
//
// One CTA owns one chunk at a time. The chunk's occupancy lives in shared memory as
// one N-bit row per (y, z) (bit x = voxel solid), plus six halo rows per side. Face
// masks of a row come from shifts of the row and its neighbours, counts from popc.
// A deterministic block scan over rows gives every row's first face; chunks of a
// batch get their global first face from a decoupled look-back over a device work
// queue. Faces are written voxel-parallel into a shared-memory staging window in the
// final byte layout and copied out with coalesced stores.
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
#include "vox_types.h"

namespace vox {

template <int N>
struct Shape {
  using RowT = typename std::conditional<(N > 32), unsigned long long, uint32_t>::type;
  static constexpr int R = N * N;                 // rows per chunk
  static constexpr int W = N > 32 ? N / 32 : 1;   // u32 words per row
  static constexpr int THREADS = N == 64 ? 512 : (N == 8 ? 64 : 256);
  static constexpr int RPT = R / THREADS;         // rows per thread in the scan
  static constexpr int LPR = N < 32 ? N : 32;     // lanes per row segment
};

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

// Shared-memory carve-up; the same function sizes the launch on the host.
template <int N, int LAYOUT>
struct SmemPlan {
  using RowT = typename Shape<N>::RowT;
  static constexpr int kTables = align16((int)sizeof(TablesDev));
  static constexpr int kOcc = align16(Shape<N>::R * (int)sizeof(RowT));
  static constexpr int kHalo = align16(6 * N * (int)sizeof(RowT));
  static constexpr int kRows = align16((Shape<N>::R + 1) * 4);
  static constexpr int kMisc = 64;
  static constexpr int kColK = align16((N + 2) * (N + 2) * 4);
  static constexpr int kFixed = kTables + kOcc + kHalo + kRows + kMisc;
  __host__ __device__ static int stage_bytes(int faces) {
    int b = LAYOUT == VOX_LAYOUT_INSTANCED ? align16(faces * 68) : faces * 96 + align16(faces * 24);
    return b < kColK ? kColK : b;
  }
  __host__ __device__ static int total(int faces) { return kFixed + stage_bytes(faces); }
};

// ------------------------------------------------------------------------------------
// Noise (Perlin improved noise, 2002) — same operation order as the CPU oracle.
// ------------------------------------------------------------------------------------

__device__ __forceinline__ float d_fade(float t) {
  return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f);
}
__device__ __forceinline__ float d_lerp(float t, float a, float b) { return a + t * (b - a); }
__device__ __forceinline__ float d_grad3(int h, float x, float y, float z) {
  h &= 15;
  float u = h < 8 ? x : y;
  float v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
  return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
__device__ __forceinline__ float d_grad2(int h, float x, float y) {
  h &= 15;
  float u = h < 8 ? x : y;
  float v = h < 4 ? y : ((h == 12 || h == 14) ? x : 0.0f);
  return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}

__device__ __forceinline__ float d_noise3(const uint8_t* p, float x, float y, float z) {
  float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  float u = d_fade(x), v = d_fade(y), w = d_fade(z);
  int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
  int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
  float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float l00 = d_lerp(u, d_grad3(p[AA], x, y, z), d_grad3(p[BA], x1, y, z));
  float l10 = d_lerp(u, d_grad3(p[AB], x, y1, z), d_grad3(p[BB], x1, y1, z));
  float l01 = d_lerp(u, d_grad3(p[AA + 1], x, y, z1), d_grad3(p[BA + 1], x1, y, z1));
  float l11 = d_lerp(u, d_grad3(p[AB + 1], x, y1, z1), d_grad3(p[BB + 1], x1, y1, z1));
  return d_lerp(w, d_lerp(v, l00, l10), d_lerp(v, l01, l11));
}

__device__ __forceinline__ float d_noise2(const uint8_t* p, float x, float y) {
  float fx = floorf(x), fy = floorf(y);
  int X = (int)fx & 255, Y = (int)fy & 255;
  x = x - fx;
  y = y - fy;
  float u = d_fade(x), v = d_fade(y);
  int A = p[X] + Y, B = p[X + 1] + Y;
  float x1 = x - 1.0f, y1 = y - 1.0f;
  float l0 = d_lerp(u, d_grad2(p[p[A]], x, y), d_grad2(p[p[B]], x1, y));
  float l1 = d_lerp(u, d_grad2(p[p[A + 1]], x, y1), d_grad2(p[p[B + 1]], x1, y1));
  return d_lerp(v, l0, l1);
}

__device__ __forceinline__ float d_fbm2(const uint8_t* p, float x, float y, const GenDev& g) {
  float sum = 0.0f, amp = 1.0f, f = g.freq;
  for (int o = 0; o < g.octaves; ++o) {
    sum = sum + amp * d_noise2(p, x * f, y * f);
    f = f * g.lac;
    amp = amp * g.gain;
  }
  return sum;
}

__device__ __forceinline__ float d_fbm3(const uint8_t* p, float x, float y, float z,
                                        const GenDev& g) {
  float sum = 0.0f, amp = 1.0f, f = g.freq;
  for (int o = 0; o < g.octaves; ++o) {
    sum = sum + amp * d_noise3(p, x * f, y * f, z * f);
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
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
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
  long long* misc;  // broadcast slots
  unsigned char* stage;
  int* colk;        // heightmap column thresholds, aliased with stage

  __device__ void carve(unsigned char* base, int stage_faces) {
    using P = SmemPlan<N, LAYOUT>;
    tab = reinterpret_cast<TablesDev*>(base);
    occ = reinterpret_cast<RowT*>(base + P::kTables);
    halo = reinterpret_cast<RowT*>(base + P::kTables + P::kOcc);
    rows = reinterpret_cast<uint32_t*>(base + P::kTables + P::kOcc + P::kHalo);
    misc = reinterpret_cast<long long*>(base + P::kTables + P::kOcc + P::kHalo + P::kRows);
    stage = base + P::kFixed;
    colk = reinterpret_cast<int*>(stage);
    (void)stage_faces;
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

// Heightmap: colk[(z+1)*(N+2) + (x+1)] = ceil(h(x, z)) - oy clamped to [-1, N + 1], so
// voxel (x, y, z) with y in [-1, N] is solid iff y < colk (== (float)(oy + y) < h).
template <int N, int LAYOUT>
__device__ void height_columns(ChunkSmem<N, LAYOUT>& s, const GenDev& g, int ox, int oy, int oz) {
  const int side = N + 2;
  for (int i = threadIdx.x; i < side * side; i += blockDim.x) {
    const int zz = i / side - 1, xx = i % side - 1;
    const bool corner = (zz < 0 || zz >= N) && (xx < 0 || xx >= N);
    int k = 0;
    if (!corner) {
      const float f = d_fbm2(s.tab->perm, (float)(ox + xx), (float)(oz + zz), g);
      const float h = g.base + g.amp * f;
      const float c = ceilf(h);
      long long kk = (long long)c - (long long)oy;
      if (!(c == c)) kk = -1;  // NaN cannot occur for finite inputs; keep it air
      k = (int)(kk < -1 ? -1 : (kk > N + 1 ? N + 1 : kk));
    }
    s.colk[i] = k;
  }
}

template <int N, int GM, int LAYOUT>
__device__ __forceinline__ bool gen_solid(const ChunkSmem<N, LAYOUT>& s, const GenDev& g, int x,
                                          int y, int z, int ox, int oy, int oz,
                                          unsigned long long s0) {
  if (GM == GM_HEIGHT) {
    return y < s.colk[(z + 1) * (N + 2) + (x + 1)];
  } else if (GM == GM_DENSITY) {
    const int wy = oy + y;
    const float f = d_fbm3(s.tab->perm, (float)(ox + x), (float)wy, (float)(oz + z), g);
    const float d = f - ((float)wy - g.y_ref) * g.y_scale;
    return g.solid_below_zero ? (d < 0.0f) : (d > 0.0f);
  } else {  // GM_BERNOULLI
    const unsigned long long i = (unsigned long long)(x + N * z + N * N * y);
    return (d_splitmix_at(s0, i) & 1ull) != 0ull;
  }
}

// Fills s.occ (own rows) and, for every set bit of `halo_mask`, the halo rows; the other
// halo rows are zero (a neighbour that is not loaded counts as air, chunk.rs:102-107).
template <int N, int GM, int LAYOUT>
__device__ void gen_chunk(ChunkSmem<N, LAYOUT>& s, const GenDev& g, vox_chunk_coord c,
                          long long chunk_index, unsigned halo_mask, bool with_halo) {
  using RowT = typename Shape<N>::RowT;
  const int ox = c.x * N, oy = c.y * N, oz = c.z * N;
  const unsigned long long s0 = g.seed ^ (unsigned long long)chunk_index;
  if (GM == GM_HEIGHT) {
    height_columns<N, LAYOUT>(s, g, ox, oy, oz);
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t* occw = reinterpret_cast<uint32_t*>(s.occ);
  for (int base = warp * 32; base < N * N * N; base += nwarps * 32) {
    const int e = base + lane;
    const int row = e / N, x = e % N;
    const int y = row / N, z = row % N;
    store_ballot<N>(occw, e, gen_solid<N, GM, LAYOUT>(s, g, x, y, z, ox, oy, oz, s0));
  }
  if (with_halo) {
    uint32_t* halow = reinterpret_cast<uint32_t*>(s.halo);
    for (int h = 0; h < 6; ++h) {
      if ((halo_mask >> h) & 1u) {
        for (int base = warp * 32; base < N * N; base += nwarps * 32) {
          const int e = base + lane;
          int x, y, z;
          halo_coord<N>(h, e / N, e % N, x, y, z);
          store_ballot<N>(halow + h * N * Shape<N>::W, e,
                          gen_solid<N, GM, LAYOUT>(s, g, x, y, z, ox, oy, oz, s0));
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

// Per-row face counts -> exclusive offsets in s.rows[0..R]; returns the chunk total.
template <int N, int LAYOUT>
__device__ uint32_t count_and_scan(ChunkSmem<N, LAYOUT>& s) {
  using RowT = typename Shape<N>::RowT;
  constexpr int RPT = Shape<N>::RPT;
  const int t = threadIdx.x;
  uint32_t cnt[RPT];
  uint32_t local = 0;
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = t * RPT + k;
    RowT m[6];
    row_masks<N, LAYOUT>(s, r / N, r % N, m);
    uint32_t c = 0;
#pragma unroll
    for (int d = 0; d < 6; ++d) c += (uint32_t)popc_row(m[d]);
    cnt[k] = c;
    local += c;
  }
  // Deterministic block scan: warp inclusive scan, then a scan of the warp totals.
  const int lane = t & 31, warp = t >> 5, nwarps = blockDim.x >> 5;
  uint32_t incl = local;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  uint32_t* wsum = reinterpret_cast<uint32_t*>(s.stage);  // scratch: staging is free here
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t v = lane < nwarps ? wsum[lane] : 0u;
    uint32_t vi = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, vi, off);
      if (lane >= off) vi += u;
    }
    if (lane < nwarps) wsum[32 + lane] = vi - v;  // exclusive warp offsets
    if (lane == nwarps - 1) wsum[64] = vi;         // chunk total
  }
  __syncthreads();
  uint32_t run = wsum[32 + warp] + incl - local;
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    s.rows[t * RPT + k] = run;
    run += cnt[k];
  }
  const uint32_t total = wsum[64];
  if (t == 0) s.rows[Shape<N>::R] = total;
  __syncthreads();
  return total;
}

// Decoupled look-back over chunks (warp 0 of the CTA). Returns the exclusive prefix of
// chunk i. Every wait is bounded; on timeout the error bit is set and 0 is used.
static __device__ unsigned long long lookback(unsigned long long* state, BatchCtl* ctl, unsigned epoch,
                                       int i, unsigned long long total) {
  const int lane = threadIdx.x & 31;
  unsigned long long excl = 0;
  if (i == 0) {
    if (lane == 0) st_relaxed_u64(&state[0], pack_state(epoch, kFlagIncl, total));
    return 0;
  }
  if (lane == 0) st_relaxed_u64(&state[i], pack_state(epoch, kFlagAgg, total));
  int j = i - 1;
  int spins = 0;
  unsigned sleep_ns = 32;
  while (true) {
    const int idx = j - lane;
    unsigned long long sv = idx >= 0 ? ld_relaxed_u64(&state[idx]) : pack_state(epoch, kFlagIncl, 0);
    const unsigned e = (unsigned)(sv >> 40) & 0xFFFFFFu;
    const unsigned long long flag = (sv >> 38) & 3ull;
    const bool valid = (e == (epoch & 0xFFFFFFu)) && flag != 0ull;
    const unsigned incl_mask = __ballot_sync(0xffffffffu, valid && flag == kFlagIncl);
    const unsigned bad_mask = __ballot_sync(0xffffffffu, !valid);
    const int first_incl = incl_mask ? __ffs(incl_mask) - 1 : 32;
    const unsigned need = first_incl >= 31 ? 0xffffffffu : ((2u << first_incl) - 1u);
    if (bad_mask & need) {
      if (++spins > kSpinLimit) {
        if (lane == 0) atomicOr(&ctl->err, ERR_TIMEOUT);
        break;
      }
      __nanosleep(sleep_ns);
      if (sleep_ns < 1024) sleep_ns <<= 1;
      continue;
    }
    unsigned long long v = (lane <= first_incl) ? (sv & ((1ull << 38) - 1)) : 0ull;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    excl += v;
    if (first_incl < 32) break;
    j -= 32;
  }
  if (lane == 0) st_relaxed_u64(&state[i], pack_state(epoch, kFlagIncl, excl + total));
  return excl;
}

// Writes face l of the staging window (chunk-local index f_local) for voxel (x, y, z).
template <int LAYOUT>
__device__ __forceinline__ void stage_face(unsigned char* stage, int stage_faces, int l, int dir,
                                           float tx, float ty, float tz, uint32_t f_local,
                                           const TablesDev* tab) {
  if (LAYOUT == VOX_LAYOUT_INSTANCED) {
    uint32_t* o = reinterpret_cast<uint32_t*>(stage + (size_t)l * 68);
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
    const float (*C)[3] = tab->corner[dir];
    const float face = __uint_as_float(tab->slot[dir]);
    const float p0x = C[0][0] + tx, p0y = C[0][1] + ty, p0z = C[0][2] + tz;
    const float p1x = C[1][0] + tx, p1y = C[1][1] + ty, p1z = C[1][2] + tz;
    const float p2x = C[2][0] + tx, p2y = C[2][1] + ty, p2z = C[2][2] + tz;
    const float p3x = C[3][0] + tx, p3y = C[3][1] + ty, p3z = C[3][2] + tz;
    v[0] = make_float4(p0x, p0y, p0z, tab->uv[0][0]);
    v[1] = make_float4(tab->uv[0][1], face, p1x, p1y);
    v[2] = make_float4(p1z, tab->uv[1][0], tab->uv[1][1], face);
    v[3] = make_float4(p2x, p2y, p2z, tab->uv[2][0]);
    v[4] = make_float4(tab->uv[2][1], face, p3x, p3y);
    v[5] = make_float4(p3z, tab->uv[3][0], tab->uv[3][1], face);
    uint2* ix = reinterpret_cast<uint2*>(stage + (size_t)stage_faces * 96 + (size_t)l * 24);
    const uint32_t b = 4u * f_local;
    ix[0] = make_uint2(b + 0u, b + 2u);
    ix[1] = make_uint2(b + 1u, b + 3u);
    ix[2] = make_uint2(b + 1u, b + 2u);
  }
}

// Copies `nw` staged faces to the global output starting at face index g.
template <int LAYOUT>
__device__ __forceinline__ void flush_stage(const unsigned char* stage, int stage_faces, int nw,
                                            unsigned long long g, void* out0, void* out1) {
  if (nw <= 0) return;
  if (LAYOUT == VOX_LAYOUT_INSTANCED) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(stage);
    uint32_t* dst = reinterpret_cast<uint32_t*>(out0) + g * 17ull;
    const int words = nw * 17;
    for (int q = threadIdx.x; q < words; q += blockDim.x) dst[q] = src[q];
  } else {
    const float4* src = reinterpret_cast<const float4*>(stage);
    float4* dst = reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(out0) + g * 96ull);
    const int v4 = nw * 6;
    for (int q = threadIdx.x; q < v4; q += blockDim.x) dst[q] = src[q];
    const uint2* isrc = reinterpret_cast<const uint2*>(stage + (size_t)stage_faces * 96);
    uint2* idst = reinterpret_cast<uint2*>(reinterpret_cast<unsigned char*>(out1) + g * 24ull);
    const int i2 = nw * 3;
    for (int q = threadIdx.x; q < i2; q += blockDim.x) idst[q] = isrc[q];
  }
}

// Emits the faces of the chunk in reference order: chunk-local face f goes to global
// face g0 + f. Windows of whole rows holding at most stage_faces faces are staged in
// shared memory and flushed with coalesced stores.
template <int N, int LAYOUT>
__device__ void emit_chunk(ChunkSmem<N, LAYOUT>& s, vox_chunk_coord c, unsigned long long g0,
                           unsigned long long cap, int stage_faces, void* out0, void* out1) {
  using RowT = typename Shape<N>::RowT;
  constexpr int R = Shape<N>::R;
  const uint32_t total = s.rows[R];
  if (total == 0) return;
  const int ox = c.x * N, oy = c.y * N, oz = c.z * N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  int r0 = 0;
  while (r0 < R) {
    const uint32_t f0 = s.rows[r0];
    if (f0 >= total) break;
    // Largest r1 with rows[r1] - f0 <= stage_faces (binary search; at least one row).
    int lo = r0 + 1, hi = R;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s.rows[mid] - f0 <= (uint32_t)stage_faces) lo = mid;
      else hi = mid - 1;
    }
    const int r1 = lo;
    const int nf = (int)(s.rows[r1] - f0);
    // Voxel-parallel staging: each lane owns one voxel of a row segment.
    const int elems = (r1 - r0) * N;
    for (int base = warp * 32; base < elems; base += nwarps * 32) {
      const int e = base + lane;
      const bool live = e < elems;
      const int r = r0 + (live ? e / N : 0);
      const int x = live ? e % N : 0;
      const int y = r / N, z = r % N;
      const uint32_t rs = s.rows[r];
      if (live && s.rows[r + 1] != rs) {
        RowT m[6];
        row_masks<N, LAYOUT>(s, y, z, m);
        const RowT below = x == 0 ? (RowT)0 : ((RowT)(~(RowT)0) >> (sizeof(RowT) * 8 - x));
        uint32_t pre = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d) pre += (uint32_t)popc_row(m[d] & below);
        int l = (int)(rs - f0 + pre);
        const float tx = (float)(ox + x), ty = (float)(oy + y), tz = (float)(oz + z);
#pragma unroll
        for (int d = 0; d < 6; ++d) {
          if ((m[d] >> x) & (RowT)1) {
            stage_face<LAYOUT>(s.stage, stage_faces, l, d, tx, ty, tz, f0 + (uint32_t)l, s.tab);
            ++l;
          }
        }
      }
    }
    __syncthreads();
    const unsigned long long g = g0 + f0;
    int nw = nf;
    if (g >= cap) nw = 0;
    else if (g + (unsigned long long)nf > cap) nw = (int)(cap - g);
    flush_stage<LAYOUT>(s.stage, stage_faces, nw, g, out0, out1);
    __syncthreads();
    r0 = r1;
  }
}

// ------------------------------------------------------------------------------------
// Kernels
// ------------------------------------------------------------------------------------

// Persistent fused generation + meshing over a device work queue (GM != GM_OCC), or
// meshing of resident occupancy (GM == GM_OCC). One chunk per CTA iteration.
template <int N, int GM, int LAYOUT>
__global__ void __launch_bounds__(Shape<N>::THREADS)
k_mesh_batch(MeshArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, LAYOUT> s;
  s.carve(smem_raw, a.stage_faces);
  load_tables<N, LAYOUT>(s, a.tables);
  __shared__ int s_item;
  __shared__ unsigned long long s_base;
  __shared__ unsigned s_epoch;
  if (threadIdx.x == 0) {
    s_epoch = ld_relaxed_u32(&a.ctl->epoch);
    __threadfence();
  }
  __syncthreads();
  const unsigned epoch = s_epoch;
  const unsigned long long words = (unsigned long long)N * N * Shape<N>::W;
  while (true) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(&a.ctl->next, 1u);
    __syncthreads();
    const int i = s_item;
    if (i >= a.n) {
      if (threadIdx.x == 0 && i == a.n + (int)gridDim.x - 1) {
        // The last ticket of this launch: reset the queue and advance the epoch.
        a.ctl->next = 0u;
        a.ctl->epoch = epoch + 1u;
      }
      break;
    }
    const vox_chunk_coord c = a.coords[i];
    if (GM == GM_OCC) {
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
      gen_chunk<N, GM, LAYOUT>(s, a.gen, c, a.index_base + i, m, true);
    }
    const uint32_t total = count_and_scan<N, LAYOUT>(s);
    if (threadIdx.x < 32) {
      const unsigned long long excl = lookback(a.state, a.ctl, epoch, i, total);
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
    emit_chunk<N, LAYOUT>(s, c, s_base, a.cap, a.stage_faces, a.out0, a.out1);
    __syncthreads();
  }
}

// Plain per-chunk mesher: one chunk, one CTA, one launch (no queue, no look-back).
template <int N, int LAYOUT>
__global__ void __launch_bounds__(Shape<N>::THREADS)
k_mesh_single(MeshArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, LAYOUT> s;
  s.carve(smem_raw, a.stage_faces);
  load_tables<N, LAYOUT>(s, a.tables);
  unsigned use = 0;
  for (int d = 0; d < 6; ++d)
    if (a.occ_nbr[d] && (d < 4 || a.full6)) use |= 1u << d;
  load_chunk<N, LAYOUT>(s, a.occ_self, a.occ_nbr, use);
  const uint32_t total = count_and_scan<N, LAYOUT>(s);
  if (threadIdx.x == 0) {
    a.face_offsets[0] = total;
    if ((unsigned long long)total > a.cap) atomicOr(&a.ctl->err, ERR_CAPACITY);
  }
  emit_chunk<N, LAYOUT>(s, a.coord_single, 0ull, a.cap, a.stage_faces, a.out0, a.out1);
}

// Chunk::new for n chunks: one CTA per chunk, occupancy rows written to global memory.
template <int N, int GM>
__global__ void __launch_bounds__(Shape<N>::THREADS)
k_generate(MeshArgs a, uint32_t* occ_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, VOX_LAYOUT_VERTEX> s;
  s.carve(smem_raw, a.stage_faces);
  load_tables<N, VOX_LAYOUT_VERTEX>(s, a.tables);
  __syncthreads();
  const int i = blockIdx.x;
  gen_chunk<N, GM, VOX_LAYOUT_VERTEX>(s, a.gen, a.coords[i], a.index_base + i, 0u, false);
  constexpr int words = N * N * Shape<N>::W;
  const uint32_t* src = reinterpret_cast<const uint32_t*>(s.occ);
  uint32_t* dst = occ_out + (size_t)i * words;
  for (int q = threadIdx.x; q < words; q += blockDim.x) dst[q] = src[q];
}

}  // namespace vox
