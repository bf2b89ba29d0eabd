// vox_raster.cu — headless rasteriser of emitted meshes (vertex layout): the reference's
// vertex stage (src/shaders/vertex.vert:22-27, gl_Position = global matrix * vertex) and
// pipeline state (src/renderer/pipeline.rs:36-45: counter-clockwise front faces, back
// faces culled, depth test Less; src/renderer/renderer.rs:92-105: clear colour
// (0.1, 0.2, 0.3), depth 1.0), with a procedural stand-in for the texture images
// (fragment.frag samples image files, which are not part of this path).
//
// Pass 1 (k_raster_tri): one thread per triangle (two per face, indices [0,2,1] and
// [3,1,2]); every covered pixel centre with depth in [0, 1) takes the 64-bit minimum of
// (depth bits << 32 | triangle id), which equals draw-order Less testing whatever the
// order the threads run in. Pass 2 (k_raster_shade): one thread per pixel shades the
// winning triangle (perspective-correct texture coordinates). Every float operation is
// written out in the order the CPU oracle uses (the file is built with -fmad=false).
#include <cstdint>

#include "voxgpu.h"
#include "vox_kernels.h"
#include "vox_types.h"

namespace vox {
namespace {

constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;

struct ScreenVert {
  float x, y, z, w;  // screen x, y (pixels, y down), NDC depth, clip w
  float u, v;
};

// Vertex k of face g through the global matrix (column-major), perspective divide and
// viewport transform. Returns false when the vertex is not in front of the camera.
__device__ __forceinline__ bool to_screen(const RasterArgs& a, unsigned long long g, int k,
                                          ScreenVert& o) {
  const float* vx = reinterpret_cast<const float*>(
      reinterpret_cast<const unsigned char*>(a.vertices) + g * 96ull + (unsigned)k * 24u);
  const float px = vx[0], py = vx[1], pz = vx[2];
  const float* m = a.m;
  const float cx = ((m[0] * px + m[4] * py) + m[8] * pz) + m[12];
  const float cy = ((m[1] * px + m[5] * py) + m[9] * pz) + m[13];
  const float cz = ((m[2] * px + m[6] * py) + m[10] * pz) + m[14];
  const float cw = ((m[3] * px + m[7] * py) + m[11] * pz) + m[15];
  if (!(cw > 0.0f)) return false;
  const float nx = cx / cw, ny = cy / cw, nz = cz / cw;
  o.x = (nx + 1.0f) * 0.5f * (float)a.width;
  o.y = (1.0f - ny) * 0.5f * (float)a.height;
  o.z = nz;
  o.w = cw;
  o.u = vx[3];
  o.v = vx[4];
  return true;
}

__device__ __forceinline__ float edge(const ScreenVert& a, const ScreenVert& b, float px, float py) {
  return (b.x - a.x) * (py - a.y) - (b.y - a.y) * (px - a.x);
}

// Top-left rule for an edge a -> b of a triangle with positive area (y down).
__device__ __forceinline__ bool top_left(const ScreenVert& a, const ScreenVert& b) {
  const float dx = b.x - a.x, dy = b.y - a.y;
  return dy < 0.0f || (dy == 0.0f && dx > 0.0f);
}

// The three vertices of triangle t of face g in the face's index order; false if culled.
__device__ __forceinline__ bool setup(const RasterArgs& a, unsigned long long g, int t,
                                      ScreenVert& v0, ScreenVert& v1, ScreenVert& v2, float& area) {
  const uint32_t* ix = reinterpret_cast<const uint32_t*>(
      reinterpret_cast<const unsigned char*>(a.indices) + g * 24ull + (unsigned)t * 12u);
  // chunk-local indices 4f + k: the vertex of this face is k = index & 3
  if (!to_screen(a, g, (int)(ix[0] & 3u), v0) || !to_screen(a, g, (int)(ix[1] & 3u), v1) ||
      !to_screen(a, g, (int)(ix[2] & 3u), v2))
    return false;
  area = edge(v0, v1, v2.x, v2.y);
  // counter-clockwise in NDC (y up) is clockwise on screen (y down): negative area
  if (!(area < 0.0f)) return false;  // back face or degenerate
  const ScreenVert tmp = v1;         // reorder to positive area
  v1 = v2;
  v2 = tmp;
  area = -area;
  return true;
}

__global__ void k_raster_clear(unsigned long long* keys, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    keys[i] = kEmptyKey;
}

__global__ void k_raster_tri(RasterArgs a, unsigned long long* keys) {
  const unsigned long long tri = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (tri >= 2ull * a.faces) return;
  ScreenVert v0, v1, v2;
  float area;
  if (!setup(a, tri >> 1, (int)(tri & 1ull), v0, v1, v2, area)) return;
  const float fx0 = fminf(fminf(v0.x, v1.x), v2.x), fx1 = fmaxf(fmaxf(v0.x, v1.x), v2.x);
  const float fy0 = fminf(fminf(v0.y, v1.y), v2.y), fy1 = fmaxf(fmaxf(v0.y, v1.y), v2.y);
  if (fx1 < 0.0f || fy1 < 0.0f || fx0 > (float)a.width || fy0 > (float)a.height) return;
  const int x0 = max(0, (int)floorf(fx0)), x1 = min(a.width - 1, (int)ceilf(fx1));
  const int y0 = max(0, (int)floorf(fy0)), y1 = min(a.height - 1, (int)ceilf(fy1));
  const bool tl0 = top_left(v1, v2), tl1 = top_left(v2, v0), tl2 = top_left(v0, v1);
  for (int py = y0; py <= y1; ++py) {
    const float sy = (float)py + 0.5f;
    for (int px = x0; px <= x1; ++px) {
      const float sx = (float)px + 0.5f;
      const float w0 = edge(v1, v2, sx, sy), w1 = edge(v2, v0, sx, sy), w2 = edge(v0, v1, sx, sy);
      const bool in = (w0 > 0.0f || (w0 == 0.0f && tl0)) && (w1 > 0.0f || (w1 == 0.0f && tl1)) &&
                      (w2 > 0.0f || (w2 == 0.0f && tl2));
      if (!in) continue;
      float z = ((w0 * v0.z + w1 * v1.z) + w2 * v2.z) / area;
      if (!(z >= 0.0f && z < 1.0f)) continue;
      z = z + 0.0f;  // -0 -> +0, so that the key order is the float order
      const unsigned long long key =
          ((unsigned long long)__float_as_uint(z) << 32) | (unsigned long long)(uint32_t)tri;
      atomicMin(keys + (size_t)py * a.width + px, key);
    }
  }
}

// Procedural texture: a base colour per texture index and a 4x4 checker over (u, v).
__device__ __forceinline__ void shade(uint32_t tex, float u, float v, uint8_t* rgba) {
  const float pal[4][3] = {{0.45f, 0.55f, 0.25f}, {0.45f, 0.32f, 0.20f},
                           {0.30f, 0.70f, 0.25f}, {0.60f, 0.60f, 0.60f}};
  const float* c = pal[tex & 3u];
  const int cu = (int)floorf(u * 4.0f), cv = (int)floorf(v * 4.0f);
  const float f = ((cu + cv) & 1) ? 0.85f : 1.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) rgba[k] = (uint8_t)(c[k] * f * 255.0f + 0.5f);
  rgba[3] = 255;
}

__global__ void k_raster_shade(RasterArgs a, const unsigned long long* keys, uint8_t* rgba) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)a.width * a.height) return;
  uint8_t* o = rgba + 4 * i;
  const unsigned long long key = keys[i];
  if (key == kEmptyKey) {  // clear colour (0.1, 0.2, 0.3, 1.0)
    o[0] = (uint8_t)(0.1f * 255.0f + 0.5f);
    o[1] = (uint8_t)(0.2f * 255.0f + 0.5f);
    o[2] = (uint8_t)(0.3f * 255.0f + 0.5f);
    o[3] = 255;
    return;
  }
  const unsigned long long tri = key & 0xFFFFFFFFull;
  const unsigned long long g = tri >> 1;
  ScreenVert v0, v1, v2;
  float area;
  setup(a, g, (int)(tri & 1ull), v0, v1, v2, area);  // the winning triangle was set up before
  const float sx = (float)(i % a.width) + 0.5f, sy = (float)(i / a.width) + 0.5f;
  const float w0 = edge(v1, v2, sx, sy), w1 = edge(v2, v0, sx, sy), w2 = edge(v0, v1, sx, sy);
  // perspective-correct interpolation: weights w_i / clip w_i
  const float b0 = w0 / v0.w, b1 = w1 / v1.w, b2 = w2 / v2.w;
  const float den = (b0 + b1) + b2;
  const float u = ((b0 * v0.u + b1 * v1.u) + b2 * v2.u) / den;
  const float v = ((b0 * v0.v + b1 * v1.v) + b2 * v2.v) / den;
  const uint32_t slot = *reinterpret_cast<const uint32_t*>(
      reinterpret_cast<const unsigned char*>(a.vertices) + g * 96ull + 20u);
  shade(a.tex[slot < 6u ? slot : 0u], u, v, o);
}

}  // namespace

cudaError_t launch_raster(const RasterArgs& a, unsigned long long* keys, uint8_t* rgba,
                          cudaStream_t st) {
  const long long px = (long long)a.width * a.height;
  k_raster_clear<<<(int)((px + 255) / 256 < 4096 ? (px + 255) / 256 : 4096), 256, 0, st>>>(keys, px);
  if (a.faces > 0) {
    const unsigned long long tris = 2ull * a.faces;
    k_raster_tri<<<(unsigned)((tris + 127) / 128), 128, 0, st>>>(a, keys);
  }
  k_raster_shade<<<(int)((px + 255) / 256), 256, 0, st>>>(a, keys, rgba);
  return cudaGetLastError();
}

}  // namespace vox
