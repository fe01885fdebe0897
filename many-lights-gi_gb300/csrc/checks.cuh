// Index checks of the bounds-checked library (built with -DMLGI_CHECKS as libmlgi_checked.so).
//
// MLGI_IX(i, n) is the index i of an access into a buffer of n elements. In the checked build an
// i outside [0, n) is recorded and replaced by 0, so that the access stays inside the buffer
// (every buffer that is accessed holds at least one element) and the kernel runs to its end; its
// results are then wrong, and the record says where. Each translation unit keeps its first
// violation since the last collection: the source line of the check (in the unit's .cu file or a
// header it includes) and the index. In the normal build MLGI_IX(i, n) is i and costs nothing.
//
// MLGI_CHECK_UNIT(name), once per translation unit, defines mlgi::checks_take_<name>, which reads
// and clears that unit's record: 0 for none, else line << 44 | the index's low 44 bits.
#pragma once

#include <cuda_runtime.h>

#ifdef MLGI_CHECKS
namespace mlgi {
namespace checks {

static __device__ unsigned long long g_first = 0ull;

static __device__ __noinline__ void record(const long long i, const int line) {
    const unsigned long long rec = ((unsigned long long)line << 44) | ((unsigned long long)i & ((1ull << 44) - 1));
    atomicCAS(&g_first, 0ull, rec);
}

template <class I>
__device__ __forceinline__ I ix(const I i, const long long n, const int line) {
    if ((unsigned long long)(long long)i < (unsigned long long)n) return i;
    record((long long)i, line);
    return I(0);
}

__device__ __forceinline__ bool range_ok(const long long first, const long long count, const long long n, const int line) {
    if (first >= 0 && count >= 0 && first + count <= n) return true;
    record(first + count - 1, line);
    return false;
}

}  // namespace checks
}  // namespace mlgi

#define MLGI_IX(i, n) ::mlgi::checks::ix((i), (long long)(n), __LINE__)
// Whether elements [first, first + count) lie in a buffer of n; records the last one when not.
#define MLGI_RANGE_OK(first, count, n) ::mlgi::checks::range_ok((long long)(first), (long long)(count), (long long)(n), __LINE__)
#define MLGI_CHECK_UNIT(name)                                                        \
    namespace mlgi {                                                                 \
    cudaError_t checks_take_##name(unsigned long long* rec) {                        \
        cudaError_t e = cudaMemcpyFromSymbol(rec, checks::g_first, sizeof(*rec));    \
        const unsigned long long zero = 0ull;                                        \
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(checks::g_first, &zero, sizeof(zero)); \
        return e;                                                                    \
    }                                                                                \
    }
#else
// (sizeof names the extents without evaluating them, so that they count as used)
#define MLGI_IX(i, n) ((void)sizeof(n), (i))
#define MLGI_RANGE_OK(first, count, n) ((void)sizeof(first), (void)sizeof(count), (void)sizeof(n), true)
#define MLGI_CHECK_UNIT(name)
#endif
