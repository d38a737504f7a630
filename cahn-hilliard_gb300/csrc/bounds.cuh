// bounds.cuh — index checks of the bounds-check build (-DCHGB_BOUNDS_CHECK;
// lib/libchgb_bc.so, built by the test that uses it).
//
// CHGB_BC(site, i, n) is true when 0 <= i < n.  In the bounds-check build a
// false one also records (site << 48) | i -- the first in this translation
// unit since the last read -- and the caller skips the access, so a bad index
// never faults; bc_read_tu reads and clears the record (chgb_bounds_report
// gathers the translation units').  In the normal build every check is the
// constant `true` and compiles away.
#pragma once

#include <cuda_runtime.h>

#ifdef CHGB_BOUNDS_CHECK
namespace chgb {
namespace {
__device__ unsigned long long bc_first;

__device__ __forceinline__ bool bc_ok(int site, long long i, long long n) {
    if(i >= 0 && i < n) return true;
    atomicCAS(&bc_first, 0ull, ((unsigned long long) (site & 0xFFFF) << 48) | ((unsigned long long) i & 0xFFFFFFFFFFFFull));
    return false;
}

inline cudaError_t bc_read_tu(unsigned long long *first) {
    cudaError_t e = cudaMemcpyFromSymbol(first, bc_first, sizeof *first);
    const unsigned long long zero = 0;
    if(e == cudaSuccess) e = cudaMemcpyToSymbol(bc_first, &zero, sizeof zero);
    return e;
}
}  // namespace
}  // namespace chgb
#define CHGB_BC(site, i, n) chgb::bc_ok((site), (long long) (i), (long long) (n))
#else
#define CHGB_BC(site, i, n) true
#endif
