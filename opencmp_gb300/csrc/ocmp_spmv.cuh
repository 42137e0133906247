// CSR SpMV building blocks shared by the assembly and Krylov translation units (sm_103a).
//
// A row is handled by TPR consecutive lanes; each lane issues U column-index and U value loads
// before any x gather, so every thread keeps up to 2U independent loads in flight, the
// memory-level parallelism the HBM-bound SpMV needs (the rows of the FE matrices here hold 7 to 60
// entries). Lanes reduce with shuffles; all TPR lanes end with the row sum.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ocmp_internal.h"

namespace ocmp {

struct RowCfg {
    int tpr, u;
};
// Threads per row and loads in flight per lane: the autotuned choice when there is one, else a
// rule on the mean row length.
inline RowCfg row_cfg(const ocmp_space_s* s) {
    if (s->tuned_tpr > 0) return {s->tuned_tpr, s->tuned_u};
    const double avg = (double)s->nnz / (double)s->ndof;
    if (avg <= 6) return {2, 4};
    if (avg <= 16) return {4, 4};
    if (avg <= 32) return {4, 8};
    if (avg <= 64) return {8, 8};
    return {16, 8};
}

template <class TM, class TV, int TPR, int U>
__device__ __forceinline__ TV row_dot(int32_t a, int32_t b, const int32_t* __restrict__ col,
                                      const TM* __restrict__ val, const TV* __restrict__ x, int lane) {
    TV acc = 0;
    for (int32_t base = a + lane; base < b; base += U * TPR) {
        int32_t c[U];
        TM v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int32_t k = base + u * TPR;
            c[u] = k < b ? __ldg(col + k) : -1;
            v[u] = k < b ? __ldg(val + k) : (TM)0;
        }
#pragma unroll
        for (int u = 0; u < U; u++)
            if (c[u] >= 0) acc += (TV)v[u] * __ldg(x + c[u]);
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPR);
    return acc;
}


}  // namespace ocmp
