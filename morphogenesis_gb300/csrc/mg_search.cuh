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

// The grid's frame: the corner of cell (0, 0, 0) and the cell extent per axis, in the
// coordinates of the particles the test is made for (a packed instance's own frame).
struct CellFrame {
    float o[3], s[3];
};

__device__ __forceinline__ CellFrame frame_of(const DevParams& P) {
    return CellFrame{{P.gmin[0], P.gmin[1], P.gmin[2]}, {P.gcell[0], P.gcell[1], P.gcell[2]}};
}

// Packed instance k: its own origin and cell extent, shifted so that the shared grid's row y
// (the instance's row y - ybase) lands where the instance's own grid has it.
__device__ __forceinline__ CellFrame frame_of(const DevParams& P, uint32_t k) {
    const InstParams& I = P.inst[k];
    return CellFrame{{I.gmin[0], I.frame_y, I.gmin[2]}, {I.gcell[0], I.gcell[1], I.gcell[2]}};
}

// Whether cell (cx, cy, cz) can hold a point of the box [b?0, b?1].  The cell's extent is
// widened by 1% of a cell on each side, far more than the rounding of the cell hash (and of a
// packed instance's shifted origin), so a point the hash put in this cell is never excluded.
__device__ __forceinline__ bool cell_meets_box(const CellFrame& f, int cx, int cy, int cz,
                                               float bx0, float bx1, float by0, float by1,
                                               float bz0, float bz1) {
    const float sx = f.s[0], sy = f.s[1], sz = f.s[2];
    const float x0 = f.o[0] + ((float)cx - 0.01f) * sx, x1 = f.o[0] + ((float)cx + 1.01f) * sx;
    const float y0 = f.o[1] + ((float)cy - 0.01f) * sy, y1 = f.o[1] + ((float)cy + 1.01f) * sy;
    const float z0 = f.o[2] + ((float)cz - 0.01f) * sz, z1 = f.o[2] + ((float)cz + 1.01f) * sz;
    return x1 >= bx0 && x0 <= bx1 && y1 >= by0 && y0 <= by1 && z1 >= bz0 && z0 <= bz1;
}

__device__ __forceinline__ bool cell_meets_box(const DevParams& P, int cx, int cy, int cz,
                                               float bx0, float bx1, float by0, float by1,
                                               float bz0, float bz1) {
    return cell_meets_box(frame_of(P), cx, cy, cz, bx0, bx1, by0, by1, bz0, bz1);
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
