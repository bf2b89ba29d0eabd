// vox_schedule.h — work-queue ticket order of the overlap schedule (host and device).
//
// The overlap kernel's CTAs draw tickets from one counter. Ticket t names a generation
// item (prepare, count and publish chunk i) or an emission item (emit segment k of a
// chunk at the offset found by look-back). The order is A(0..L-1), then A(L+m) and C(m)
// alternately while generation items remain, then the remaining emission items, so the
// chunk of every emission item, and every chunk before it, has a smaller ticket than the
// item: an item only ever waits for work that a running CTA holds or has finished.
// Plain C++ as well, so that host tests check the order itself.
#pragma once

#ifdef __CUDACC__
#define VOX_HD __host__ __device__ __forceinline__
#else
#define VOX_HD inline
#endif

namespace vox {

// Item of ticket t: returns 0 (generation, idx = chunk), 1 (emission, idx = item) or 2
// (past the end). n chunks, `items` emission items (>= n), lag L in [0, n].
VOX_HD int overlap_ticket(unsigned t, unsigned n, unsigned items, unsigned L, unsigned& idx) {
  if (t < L) {
    idx = t;
    return 0;
  }
  const unsigned P = n - L;  // interleaved pairs
  const unsigned u = t - L;
  if (u < 2u * P) {
    idx = (u & 1u) ? (u >> 1) : L + (u >> 1);
    return (u & 1u) ? 1 : 0;
  }
  idx = P + (u - 2u * P);
  return idx < items ? 1 : 2;
}

}  // namespace vox
