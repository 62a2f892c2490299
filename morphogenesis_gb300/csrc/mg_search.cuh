// mg_search.cuh - pieces of the warp-cooperative neighbour search shared by the density pass
// and the re-forming search: the 27-cell window of a cell, warp reductions, the candidate
// prefilter distance and the cell-box test.
#pragma once
#include "mg_internal.cuh"

namespace mg {

struct CellWin {
    int x, y, z;  // window origin = own cell - (1,1,1)
};

__device__ __forceinline__ CellWin window_of(const DevParams& P, uint32_t cell) {
    CellWin w;
    w.x = (int)(cell % (uint32_t)P.res[0]) - 1;
    w.z = (int)((cell / (uint32_t)P.res[0]) % (uint32_t)P.res[2]) - 1;
    w.y = (int)(cell / ((uint32_t)P.res[0] * (uint32_t)P.res[2])) - 1;
    return w;
}


__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, d));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, d));
    return v;
}

// Squared distance with fused multiply-adds: within a few ulps of the reference expression,
// used only to choose list candidates.
__device__ __forceinline__ float approx_dsq(float4 a, float4 b) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Whether cell (cx, cy, cz) can hold a point of the box [b?0, b?1].  The cell's extent is
// widened by 1% of a cell on each side, far more than the rounding of the cell hash, so a
// point the hash put in this cell is never excluded.
__device__ __forceinline__ bool cell_meets_box(const DevParams& P, int cx, int cy, int cz,
                                               float bx0, float bx1, float by0, float by1,
                                               float bz0, float bz1) {
    const float sx = P.gcell[0], sy = P.gcell[1], sz = P.gcell[2];
    const float x0 = P.gmin[0] + ((float)cx - 0.01f) * sx, x1 = P.gmin[0] + ((float)cx + 1.01f) * sx;
    const float y0 = P.gmin[1] + ((float)cy - 0.01f) * sy, y1 = P.gmin[1] + ((float)cy + 1.01f) * sy;
    const float z0 = P.gmin[2] + ((float)cz - 0.01f) * sz, z1 = P.gmin[2] + ((float)cz + 1.01f) * sz;
    return x1 >= bx0 && x0 <= bx1 && y1 >= by0 && y0 <= by1 && z1 >= bz0 && z0 <= bz1;
}

__device__ __forceinline__ int warp_mini(int v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, d));
    return v;
}
__device__ __forceinline__ int warp_maxi(int v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, d));
    return v;
}

}  // namespace mg
