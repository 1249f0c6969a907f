// Slot bookkeeping of the TMA tile rings in hs2g_lines.cu, kept apart from the kernels so that it compiles as
// plain C++ and is checked on the host (tests/test_ring_bookkeeping.py).
//
// A ring has up to 32 slots; each slot's copies complete on the slot's mbarrier, whose phase alternates.  The
// producer marks a slot pending when it issues copies into it.  A wait that saw the phase complete advances
// the slot (flips its expected phase, clears pending); a wait that gave up (bounded wait, timed out) leaves
// both as they were, so that the abort path still knows which copies are in flight and on which phase to
// wait for them before the CTA exits.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define HS2G_HD __host__ __device__ __forceinline__
#else
#define HS2G_HD inline
#endif

namespace hs2g {

struct SlotRing {
  uint32_t parity = 0;   // bit s: phase of the next completion of slot s
  uint32_t pending = 0;  // bit s: copies issued into slot s and not yet seen complete

  HS2G_HD uint32_t phase(int s) const { return (parity >> s) & 1u; }
  HS2G_HD void issued(int s) { pending |= 1u << s; }
  HS2G_HD void waited(int s, bool completed) {
    if (completed) {
      parity ^= 1u << s;
      pending &= ~(1u << s);
    }
  }
  HS2G_HD bool in_flight(int s) const { return ((pending >> s) & 1u) != 0; }
};

}  // namespace hs2g
