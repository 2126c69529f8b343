// scatter.cuh — grouped vector reductions of the scatter back projection
// (bp[col] += val · ratio[row], calcBwProj_none_trans, kernel.cu:165-177),
// shared by the scatter kernel (spmv.cu) and the fused single pass
// (spmv_fused.cu).
#pragma once

#include "common.cuh"

namespace mlem {

// One 16-byte reduction into bp[4g .. 4g+3]: red.global.add.v4.f32 (one L2
// atomic operation for four floats) where the group lies inside bp and bp is
// 16-byte aligned (a caller's output pointer may not be), else the components
// that carry a product one by one.
__device__ __forceinline__ void red_group(float* __restrict__ bp, uint32_t ncols, uint32_t g, const float a[4],
                                          unsigned used) {
    const uint32_t c0 = g << 2;
    if (c0 + 3 < ncols && (reinterpret_cast<uintptr_t>(bp) & 15u) == 0) {
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(bp + c0), "f"(a[0]), "f"(a[1]),
                     "f"(a[2]), "f"(a[3])
                     : "memory");
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (used & (1u << j)) atomicAdd(bp + c0 + j, a[j]);
    }
}

// Scatters the products p[k] of four consecutive entries (those whose bit k
// is set in `use`) into bp.  Within a row the columns ascend, so entries whose
// columns share a 16-byte group (column >> 2) are adjacent: each group goes
// out as one vector reduction, with zeros in its unused components (adding
// +0.0 leaves a sum unchanged).  Entries of one group are summed first.  Where
// the four entries span two rows the group changes at the row boundary and
// the reductions stay correct.  In the 3-D scanners about 0.6 reductions are
// issued per nonzero instead of 1.
__device__ __forceinline__ void scatter4_mask(float* __restrict__ bp, uint32_t ncols, const uint4& c,
                                              const float p[4], unsigned use) {
    const uint32_t cs[4] = {c.x, c.y, c.z, c.w};
    float a[4] = {0.f, 0.f, 0.f, 0.f};
    unsigned used = 0;
    uint32_t grp = 0xffffffffu;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!(use & (1u << k))) continue;
        const uint32_t g = cs[k] >> 2, j = cs[k] & 3u;
        if (g != grp) {
            if (used) red_group(bp, ncols, grp, a, used);
            a[0] = a[1] = a[2] = a[3] = 0.f;
            used = 0;
            grp = g;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (j == (uint32_t)q) a[q] = __fadd_rn(a[q], p[k]);
        used |= 1u << j;
    }
    if (used) red_group(bp, ncols, grp, a, used);
}

}  // namespace mlem
