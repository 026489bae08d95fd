// Index checks of the debug build (compiled with FDTDPIC_BOUNDS_CHECK: libfdtdpic_bounds.so).
// FDTD_IN(i, n, status) is true when 0 <= i < n; otherwise it raises FDTD_STATUS_BOUNDS in
// *status (when status is not NULL) and is false, and the caller skips the access instead of
// touching memory outside the buffer.  In the release build FDTD_IN is the constant true and
// compiles away: there the same indices are kept in range by construction (particles outside
// the grid are counted and skipped, deposit windows and segments are checked against their
// sizes), which is what the debug build verifies.
#pragma once
#include <stdint.h>

#include "fdtdpic.h"

#ifdef FDTDPIC_BOUNDS_CHECK
__device__ __forceinline__ bool fdtd_in_range(long long i, long long n, int32_t *status)
{
    if (i >= 0 && i < n) return true;
    if (status) atomicOr(status, FDTD_STATUS_BOUNDS);
    return false;
}
#define FDTD_IN(i, n, status) fdtd_in_range((long long)(i), (long long)(n), (status))
#else
#define FDTD_IN(i, n, status) true
#endif
