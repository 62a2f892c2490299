// mg_mlp.cu - training and inference kernels of the learned reaction surrogate (row a12).
//
// Training: BF16 GEMMs on 5th-generation tensor cores (tcgen05.mma, FP32 accumulators in
// tensor memory, split-K for the weight gradients) for the forward and backward products,
// elementwise bias/GELU/loss kernels and Adam on FP32 master weights.
// Inference (inside the simulation step): one persistent kernel per SM that runs the three
// layers on 5th-generation tensor cores -- tcgen05.mma with operands in shared memory
// (K-major core-matrix layout, no swizzle) and FP32 accumulators in tensor memory, read back
// with tcgen05.ld for the bias + GELU epilogue.  Every wait on the MMA-completion mbarrier is
// bounded; on timeout the kernel records MLP_ERR_MBAR_TIMEOUT, frees its tensor memory and
// returns.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mg_internal.cuh"
#include "mg_mlp.cuh"

namespace mg {

using bf16 = __nv_bfloat16;

// =============================================================================================
// Training elementwise kernels
// =============================================================================================
// Batch assembly: rows drawn uniformly (with replacement) from the dataset by a counter-based
// hash of (seed, step, row); features and targets normalised; features rounded to bf16.
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27; x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__global__ void k_make_batch(const float* __restrict__ dx, const float* __restrict__ dy,
                             uint64_t nrows, uint32_t B, uint64_t seed, const float* __restrict__ norm,
                             bf16* __restrict__ X, float* __restrict__ Y, int sequential) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint64_t row = sequential ? (uint64_t)b % nrows
                                    : mix64(seed ^ (0x9e3779b97f4a7c15ull * (b + 1))) % nrows;
    const float* mx = norm, *sx = norm + MLP_IN, *my = norm + 2 * MLP_IN, *sy = my + MLP_OUT;
    for (int i = 0; i < MLP_IN; i++)
        X[(size_t)b * MLP_IN + i] = __float2bfloat16((dx[row * MLP_IN + i] - mx[i]) * sx[i]);
    for (int o = 0; o < MLP_OUT; o++)
        Y[(size_t)b * MLP_OUT + o] = (dy[row * MLP_OUT + o] - my[o]) * sy[o];
}

// Z += bias; optionally H = bf16(gelu(Z)).
__global__ void k_bias_act(float* __restrict__ Z, const float* __restrict__ bias, int O, size_t n,
                           bf16* __restrict__ H) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float z = Z[e] + bias[e % O];
    Z[e] = z;
    if (H) H[e] = __float2bfloat16(gelu(z));
}

// d(mean squared error)/dY and the loss sum.
__global__ void k_out_grad(const float* __restrict__ Yp, const float* __restrict__ Y, size_t n,
                           float scale, bf16* __restrict__ dY16, float* __restrict__ dY32,
                           double* __restrict__ loss) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (e < n) {
        const float d = Yp[e] - Y[e];
        const float gr = 2.f * d * scale;
        dY16[e] = __float2bfloat16(gr);
        dY32[e] = gr;
        l = d * d;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) l += __shfl_xor_sync(0xffffffffu, l, s);
    if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, (double)l);
}

// dZ = dH * gelu'(Z) (fp32 and bf16 copies).
__global__ void k_act_grad(const float* __restrict__ dH, const float* __restrict__ Z, size_t n,
                           bf16* __restrict__ dZ16, float* __restrict__ dZ32) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float v = dH[e] * gelu_grad(Z[e]);
    dZ16[e] = __float2bfloat16(v);
    dZ32[e] = v;
}

// db[o] += sum_b dZ[b][o]
__global__ void k_colsum(const float* __restrict__ dZ, int rows, int O, float* __restrict__ db) {
    const int o = blockIdx.x;
    float s = 0.f;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) s += dZ[(size_t)r * O + o];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[o] = red[0];
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = gr[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_to_bf16(const float* __restrict__ src, bf16* __restrict__ dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16(src[i]);
}

// Column statistics of the dataset for the normalisation: sums and sums of squares.
__global__ void k_col_stats(const float* __restrict__ d, uint64_t rows, int cols,
                            double* __restrict__ acc) {
    const int c = blockIdx.y;
    double s = 0.0, s2 = 0.0;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const double x = d[r * cols + c];
        s += x;
        s2 += x * x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[2 * c], s);
        atomicAdd(&acc[2 * c + 1], s2);
    }
}

// =============================================================================================
// Inference on tcgen05
// =============================================================================================
// One CTA per SM holding the weights once, with INF_GROUPS independent groups of warps, each
// with its own 128-particle tile in flight (activation buffer, TMEM columns, mbarrier): while
// one group runs its GELU epilogue the tensor core works on another group's layer.  In a group,
// warp w reads TMEM lanes 32(w%4)..32(w%4)+31 (its tile rows) and, in the hidden-layer
// epilogues, the w/4-th of the INF_SPLIT column ranges of its group's 128.
#ifndef MG_INF_GROUPS
#define MG_INF_GROUPS 4
#endif
#ifndef MG_INF_SPLIT
#define MG_INF_SPLIT 2
#endif
constexpr int INF_GROUPS = MG_INF_GROUPS;
constexpr int INF_SPLIT = MG_INF_SPLIT;                // threads per tile row (1 or 2)
constexpr int INF_GROUP_THREADS = 128 * INF_SPLIT;
constexpr int INF_THREADS = INF_GROUPS * INF_GROUP_THREADS;
constexpr uint32_t INF_COLS = MLP_H / INF_SPLIT;       // hidden columns per thread
static_assert(INF_GROUPS * 128 <= 512, "TMEM columns of the groups");
constexpr int INF_TMEM_COLS = 512;  // allocation (power of two); groups use 128 columns each
constexpr uint32_t MBAR_SPIN_LIMIT = 1u << 24;

struct InferSmem {
    bf16 w1[MLP_H * MLP_IN];    // 12 KB  B operand layer 1 (N=128 x K=48)
    bf16 w2[MLP_H * MLP_H];     // 32 KB  B operand layer 2 (N=128 x K=128)
    bf16 w3[MLP_OUT * MLP_H];   //  4 KB  B operand layer 3 (N=16 x K=128)
    // per group: A operand of layer 1, the tile's 128 x 48 features as six TMA planes of 8
    // features x 128 rows (2 KB each: plane kb holds core matrices (row group, kb) 128 bytes
    // apart), loaded one tile ahead
    bf16 feat[INF_GROUPS][128 * MLP_IN];
    // per group: A operand of layers 2 and 3 (128 x 128, core-matrix layout)
    bf16 act[INF_GROUPS][128 * MLP_H];
    alignas(16) float b1[MLP_H];
    alignas(16) float b2[MLP_H];
    alignas(16) float b3[MLP_OUT];
    unsigned long long mbar[INF_GROUPS];  // MMA completion
    unsigned long long tbar[INF_GROUPS];  // feature tile arrival (TMA transaction bytes)
    uint32_t tmem_base;
};
static_assert(sizeof(InferSmem) <= 232448, "inference shared memory above the 227 KB a CTA may use");
constexpr uint32_t FEAT_PLANE_BYTES = 128u * 8u * 2u;               // 8 features x 128 rows
constexpr uint32_t FEAT_TILE_BYTES = FEAT_PLANE_BYTES * (MLP_IN / 8);  // 12 KB

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension byte offset
// (K direction: next core matrix along K), stride-dimension byte offset (M/N direction: next
// group of 8 rows), version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;  // descriptor version for tcgen05
    return d;                 // base offset 0, relative LBO, swizzle mode 0 (none)
}

// Instruction descriptor of kind::f16: D = F32, A = B = BF16, both K-major, dense.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
    return (1u << 4)            // D format F32
           | (1u << 7)          // A format BF16
           | (1u << 10)         // B format BF16
           | ((N >> 3) << 17)   // N / 8
           | ((M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_f16_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                           uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar_saddr) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     mbar_saddr)
                 : "memory");
}

// Bounded parity wait; returns false when the wait gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar_saddr, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; it++) {
        uint32_t done = 0;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar_saddr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 32 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// Writes 8 consecutive bf16 of row r, columns k..k+7, into a rows x K core-matrix tile.
__device__ __forceinline__ void put8(bf16* tile, uint32_t r, uint32_t k, uint32_t K,
                                     const float (&v)[8]) {
    __nv_bfloat162 h[4];
#pragma unroll
    for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4*>(tile + core_offset(r, k, K)) = *reinterpret_cast<uint4*>(h);
}

#ifndef MG_MLP_PACKED
#define MG_MLP_PACKED 1
#endif
// bias + GELU of eight accumulator columns (biases b[0..7], 16-byte aligned in shared memory):
// the gelu() expression with two columns per packed f32x2 operation, the tanh per column
__device__ __forceinline__ void bias_gelu8(const float* v, const float* b, float (&h)[8]) {
#if MG_MLP_PACKED
    const float4 b0 = *reinterpret_cast<const float4*>(b), b4 = *reinterpret_cast<const float4*>(b + 4);
    const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b4.x, b4.y, b4.z, b4.w};
    const float2 k01 = make_float2(GELU_K0 * GELU_K1, GELU_K0 * GELU_K1), k0 = make_float2(GELU_K0, GELU_K0);
    const float2 half = make_float2(0.5f, 0.5f);
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        const float2 x = __fadd2_rn(make_float2(v[i], v[i + 1]), make_float2(bb[i], bb[i + 1]));
        const float2 u = __fmul2_rn(x, __ffma2_rn(k01, __fmul2_rn(x, x), k0));
        const float2 hx = __fmul2_rn(half, x);
        const float2 r = __ffma2_rn(hx, make_float2(tanh_hw(u.x), tanh_hw(u.y)), hx);
        h[i] = r.x;
        h[i + 1] = r.y;
    }
#else
#pragma unroll
    for (int i = 0; i < 8; i++) h[i] = gelu(v[i] + b[i]);
#endif
}

// One feature tile (rows row0 .. row0 + 127, all 48 features) into its six planes: the
// mbarrier expects the tile's bytes, and each TMA load of a plane completes its share (rows
// past the matrix read as zeros).  The planes start at feature 0, 8, ..., 40 (16-byte aligned
// x coordinates).  Single thread.
__device__ __forceinline__ void feat_tile_tma(bf16* planes, const CUtensorMap* map, uint32_t row0,
                                              uint32_t bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(FEAT_TILE_BYTES)
                 : "memory");
#pragma unroll
    for (uint32_t kb = 0; kb < MLP_IN / 8; kb++)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
            "[%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_u32(planes + kb * 128u * 8u)),
            "l"(reinterpret_cast<uint64_t>(map)), "r"(kb * 8u), "r"(row0), "r"(bar)
            : "memory");
}

// Layer 1 from the feature planes: D[128 x 128] = F[128 x 48] * W1[128 x 48]^T.  In the planes
// the two core matrices of a K=16 step are a plane apart (leading byte offset 2 KB) and row
// groups 128 bytes apart (stride byte offset); W1 keeps the core-matrix tile layout.
__device__ __forceinline__ void issue_layer1(uint32_t d_tmem, const bf16* planes, const bf16* w1) {
    const uint32_t sa = smem_u32(planes), sb = smem_u32(w1);
    const uint32_t idesc = idesc_bf16(128, MLP_H);
#pragma unroll
    for (uint32_t s = 0; s < MLP_IN / 16; s++) {
        const uint64_t ad = smem_desc(sa + s * 2u * FEAT_PLANE_BYTES, FEAT_PLANE_BYTES, 128u);
        const uint64_t bd = smem_desc(sb + s * 256u, 128u, (MLP_IN >> 3) * 128u);
        mma_f16_ss(d_tmem, ad, bd, idesc, s > 0 ? 1u : 0u);
    }
}

// Issues one layer: D[128 x N] = A[128 x K] * B[N x K]^T, K/16 MMAs (single thread).
__device__ __forceinline__ void issue_layer(uint32_t d_tmem, const bf16* a, const bf16* b, uint32_t K,
                                            uint32_t N) {
    const uint32_t sa = smem_u32(a), sb = smem_u32(b);
    const uint32_t sbo = (K >> 3) * 128u;  // next group of 8 rows
    const uint32_t idesc = idesc_bf16(128, N);
    for (uint32_t s = 0; s < K / 16; s++) {
        const uint64_t ad = smem_desc(sa + s * 256u, 128u, sbo);
        const uint64_t bd = smem_desc(sb + s * 256u, 128u, sbo);
        mma_f16_ss(d_tmem, ad, bd, idesc, s > 0 ? 1u : 0u);
    }
}

// Named barrier of one warp group (ids 1..INF_GROUPS; 0 is __syncthreads).
__device__ __forceinline__ void group_sync(uint32_t g) {
    asm volatile("bar.sync %0, %1;\n" ::"r"(g + 1u), "r"((uint32_t)INF_GROUP_THREADS) : "memory");
}
// AND of a predicate over one warp group (a barrier too).
__device__ __forceinline__ bool group_and(uint32_t g, bool v) {
    uint32_t out;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, %2, %3, q;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(out)
        : "r"((uint32_t)v), "r"(g + 1u), "r"((uint32_t)INF_GROUP_THREADS)
        : "memory");
    return out != 0;
}

// =============================================================================================
// Training GEMM on tcgen05: C (+)= sum_k A(m, k) B(n, k), BF16 operands, FP32 accumulators
// =============================================================================================
// A(m, k) = A.p[m * A.s_row + k * A.s_k], B(n, k) = B.p[n * B.s_row + k * B.s_k], C(m, n) at
// C[m * scm + n * scn].  One CTA of 128 threads computes a 128 x nt tile (nt = the tile's
// columns rounded up to 16, at most 128) over one K range of a split-K grid (atomicAdd into C
// when split > 1).  The threads stage 64-wide K chunks of both operands into shared memory in
// the K-major core-matrix layout (transposing 8 x 8 blocks in registers when the operand is
// contiguous along its rows rather than along K), double-buffered: one elected thread issues
// the chunk's four tcgen05.mma (M 128, K 16 each) and commits them to the buffer's mbarrier
// while the others stage the next chunk.  The accumulator lives in 128 TMEM columns; warp w
// reads lanes 32w..32w+31 (rows) back with tcgen05.ld.  Every mbarrier wait is bounded: on
// timeout the CTA records MLP_ERR_MBAR_TIMEOUT, waits (bounded) for its MMAs in flight, frees
// its tensor memory and returns.
constexpr int TG_BM = 128, TG_BN = 128, TG_BK = 64, TG_THREADS = 128;
constexpr uint32_t TG_TMEM_COLS = 128;

struct GemmOperand {
    const bf16* p;
    long s_row, s_k;
    int mode;  // 1: K contiguous (16-byte loads), 0: rows contiguous (8 x 8 transposes), -1: scalar
};

struct GemmSmem {
    bf16 a[2][TG_BM * TG_BK];  // 16 KB per buffer
    bf16 b[2][TG_BN * TG_BK];  // 16 KB per buffer
    unsigned long long mbar[2];
    uint32_t tmem_base;
};

__device__ __forceinline__ bf16 gemm_elem(const GemmOperand& o, int r, int k, int rows, int kend) {
    return (r < rows && k < kend) ? o.p[(long)r * o.s_row + (long)k * o.s_k] : __float2bfloat16(0.f);
}

// Rows [row0, row0 + nrows) x K [k0, k0 + TG_BK) of an operand into a core-matrix tile; zeros
// at rows >= rows_lim and at k >= kend.
__device__ __forceinline__ void gemm_stage(bf16* tile, const GemmOperand& o, int row0, int rows_lim,
                                           int nrows, int k0, int kend, int tid) {
    if (o.mode == 1) {
        for (int idx = tid; idx < nrows * (TG_BK / 8); idx += TG_THREADS) {
            const int r = idx >> 3, kq = (idx & 7) * 8, gr = row0 + r, gk = k0 + kq;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gr < rows_lim) {
                if (gk + 8 <= kend) {
                    v = *reinterpret_cast<const uint4*>(o.p + (long)gr * o.s_row + gk);
                } else {
                    bf16 e[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) e[j] = gemm_elem(o, gr, gk + j, rows_lim, kend);
                    v = *reinterpret_cast<uint4*>(e);
                }
            }
            *reinterpret_cast<uint4*>(tile + core_offset(r, kq, TG_BK)) = v;
        }
    } else if (o.mode == 0) {
        // one 8 x 8 block (one core matrix) per thread and pass: eight 16-byte loads along the
        // rows, one per k, transposed into eight 16-byte rows along k
        for (int idx = tid; idx < (nrows / 8) * (TG_BK / 8); idx += TG_THREADS) {
            const int r0 = (idx >> 3) * 8, kq = (idx & 7) * 8, gr0 = row0 + r0;
            uint32_t w[8][4];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int gk = k0 + kq + j;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (gk < kend) {
                    if (gr0 + 8 <= rows_lim) {
                        v = *reinterpret_cast<const uint4*>(o.p + (long)gk * o.s_k + gr0);
                    } else {
                        bf16 e[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) e[i] = gemm_elem(o, gr0 + i, gk, rows_lim, kend);
                        v = *reinterpret_cast<uint4*>(e);
                    }
                }
                w[j][0] = v.x; w[j][1] = v.y; w[j][2] = v.z; w[j][3] = v.w;
            }
#pragma unroll
            for (int i = 0; i < 8; i++) {
                // row i: element i of each k, two k per 32-bit word (the lower k in the low half)
                const uint32_t sel = (i & 1) ? 0x7632u : 0x5410u;
                uint4 out;
                out.x = __byte_perm(w[0][i >> 1], w[1][i >> 1], sel);
                out.y = __byte_perm(w[2][i >> 1], w[3][i >> 1], sel);
                out.z = __byte_perm(w[4][i >> 1], w[5][i >> 1], sel);
                out.w = __byte_perm(w[6][i >> 1], w[7][i >> 1], sel);
                *reinterpret_cast<uint4*>(tile + core_offset(r0 + i, kq, TG_BK)) = out;
            }
        }
    } else {
        for (int idx = tid; idx < nrows * TG_BK; idx += TG_THREADS) {
            const int r = idx / TG_BK, k = idx % TG_BK;
            tile[core_offset(r, k, TG_BK)] = gemm_elem(o, row0 + r, k0 + k, rows_lim, kend);
        }
    }
}

__global__ void __launch_bounds__(TG_THREADS) k_gemm_tc(int M, int N, int K, GemmOperand A, GemmOperand B,
                                                        float* __restrict__ C, long scm, long scn, int split,
                                                        uint32_t* __restrict__ err, uint32_t spin_limit,
                                                        uint32_t withhold) {
    // withhold != 0 (failure-detection self-test only) issues no MMA, so a wait runs out
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    GemmSmem& S = *reinterpret_cast<GemmSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * TG_BM, n0 = blockIdx.x * TG_BN;
    const int ncols = min(TG_BN, N - n0);
    const uint32_t nt = (uint32_t)((ncols + 15) & ~15);
    const int per = ((K + split - 1) / split + TG_BK - 1) / TG_BK * TG_BK;
    const int kb = blockIdx.z * per, ke = min(K, kb + per);
    const int nchunks = ke > kb ? (ke - kb + TG_BK - 1) / TG_BK : 0;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.mbar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.mbar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_u32(&S.tmem_base)),
                     "r"(TG_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    bool ok = true;
    int issued = 0;  // chunks committed (thread 0)
    for (int c = 0; c < nchunks; c++) {
        const int buf = c & 1;
        if (c >= 2) {  // the MMAs of chunk c - 2 have finished reading this buffer
            ok = __syncthreads_and(mbar_wait(smem_u32(&S.mbar[buf]), ((c - 2) >> 1) & 1, spin_limit));
            if (!ok) break;
            tc_fence_after();
        }
        const int k0 = kb + c * TG_BK;
        gemm_stage(S.a[buf], A, m0, M, TG_BM, k0, ke, tid);
        gemm_stage(S.b[buf], B, n0, N, (int)nt, k0, ke, tid);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0 && !withhold) {
            const uint32_t sa = smem_u32(S.a[buf]), sb = smem_u32(S.b[buf]);
            const uint32_t sbo = (TG_BK >> 3) * 128u;  // next group of 8 rows
            const uint32_t idesc = idesc_bf16(TG_BM, nt);
#pragma unroll
            for (uint32_t s = 0; s < TG_BK / 16; s++)
                mma_f16_ss(tmem, smem_desc(sa + s * 256u, 128u, sbo), smem_desc(sb + s * 256u, 128u, sbo),
                           idesc, (c > 0 || s > 0) ? 1u : 0u);
            mma_commit(smem_u32(&S.mbar[buf]));
            issued = c + 1;
        }
    }
    if (ok && nchunks > 0) {
        // the last two chunks (the earlier ones were waited for in the loop)
        const int l = nchunks - 1;
        bool w = mbar_wait(smem_u32(&S.mbar[l & 1]), (l >> 1) & 1, spin_limit);
        if (w && l > 0) w = mbar_wait(smem_u32(&S.mbar[(l - 1) & 1]), ((l - 1) >> 1) & 1, spin_limit);
        ok = __syncthreads_and(w);
        if (ok) {
            tc_fence_after();
            const int gm = m0 + warp * 32 + lane;
            const uint32_t taddr = tmem + (((uint32_t)warp * 32u) << 16);
            const bool vec = split == 1 && scn == 1 && (scm & 3) == 0 &&
                             ((reinterpret_cast<uintptr_t>(C) & 15u) == 0) && ((n0 & 3) == 0);
            for (uint32_t c0 = 0; c0 < nt; c0 += 16) {
                float v[16];
                tmem_ld16(taddr + c0, v);
                if (gm < M) {
                    const int nb = n0 + (int)c0;
                    float* row = C + (long)gm * scm;
                    if (vec && (int)c0 + 16 <= ncols) {
                        float4* o = reinterpret_cast<float4*>(row + nb);
#pragma unroll
                        for (int q = 0; q < 4; q++) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    } else {
#pragma unroll
                        for (int j = 0; j < 16; j++) {
                            if ((int)c0 + j < ncols) {
                                float* d = row + (long)(nb + j) * scn;
                                if (split > 1) atomicAdd(d, v[j]);
                                else *d = v[j];
                            }
                        }
                    }
                }
            }
        }
    }
    if (!ok && tid == 0) {
        atomicOr(err, MLP_ERR_MBAR_TIMEOUT);
        if (issued > 0)  // one more bounded wait for the MMAs in flight before the TMEM is freed
            mbar_wait(smem_u32(&S.mbar[(issued - 1) & 1]), ((issued - 1) >> 1) & 1, spin_limit);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(S.tmem_base),
                     "r"(TG_TMEM_COLS)
                     : "memory");
}

GemmOperand gemm_operand(const bf16* p, long s_row, long s_k) {
    const bool aligned = (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
    int mode = -1;
    if (aligned && s_k == 1 && s_row % 8 == 0) mode = 1;
    else if (aligned && s_row == 1 && s_k % 8 == 0) mode = 0;
    return GemmOperand{p, s_row, s_k, mode};
}

// C(m, n) (+)= sum_k A(m, k) B(k, n) with A(m, k) = A[m*sam + k*sak], B(k, n) = B[k*sbk + n*sbn]
// (bf16), C(m, n) at C[m*ldc + n] (fp32).  K split over gridDim.z with atomic accumulation
// when split > 1 (C must then be zeroed first).  A product with fewer than 64 rows runs
// transposed (C^T = B^T A^T) so that the 128-row MMA tile is filled by the longer side.
void launch_gemm_bf16(int M, int N, int K, const bf16* A, long sam, long sak, const bf16* B,
                      long sbk, long sbn, float* C, long ldc, int split, uint32_t* err, cudaStream_t st,
                      uint32_t withhold = 0) {
    GemmOperand a = gemm_operand(A, sam, sak), b = gemm_operand(B, sbn, sbk);
    long scm = ldc, scn = 1;
    if (M < 64 && N > M) {
        std::swap(a, b);
        std::swap(M, N);
        std::swap(scm, scn);
    }
    dim3 grid((N + TG_BN - 1) / TG_BN, (M + TG_BM - 1) / TG_BM, split);
    k_gemm_tc<<<grid, TG_THREADS, sizeof(GemmSmem), st>>>(M, N, K, a, b, C, scm, scn, split, err,
                                                          MBAR_SPIN_LIMIT, withhold);
}

// Surrogate step: for each particle p < nactive, conc_out[p] = conc_in[p] + s_p * MLP(features[p])
// (s_p the particle's input scale, 1 without feat_scale).  Particles under judgement (sampled
// this step) or already handed to the plain method (bit 31 of their gene word) compare against /
// take the plain update in conc_plain.
__global__ void __launch_bounds__(INF_THREADS, 1) k_mlp_infer(
    InferWeights W, const __grid_constant__ CUtensorMap feat_map, const float* __restrict__ feat_scale,
    const float* conc_in,
    const float* __restrict__ conc_plain, float* conc_out, uint32_t* __restrict__ genes,
    const uint32_t* __restrict__ nactive_p, uint32_t ntotal_override, const uint32_t* __restrict__ step_p,
    uint32_t judge_period, uint32_t judge_stride, float threshold, uint32_t* __restrict__ stats,
    uint32_t* __restrict__ err, uint32_t spin_limit, uint32_t withhold) {
    // spin_limit bounds every wait (feature arrival, MMA completion); withhold != 0
    // (failure-detection self-test only) issues no MMA, so the first completion wait runs out
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t g = tid / INF_GROUP_THREADS;            // warp group
    const uint32_t gtid = tid % INF_GROUP_THREADS;         // thread in the group
    const uint32_t gwarp = gtid >> 5;
    const uint32_t n = nactive_p ? *nactive_p : ntotal_override;
    const uint32_t step = step_p ? *step_p : 0u;
    const bool judge_step = judge_period && judge_stride && (step % judge_period) == 0;
    const uint32_t judge_phase = judge_step ? (step / judge_period) % judge_stride : 0u;

    // weights and biases into shared memory (already in the core-matrix layout)
    {
        const uint4* s1 = reinterpret_cast<const uint4*>(W.w1);
        uint4* d1 = reinterpret_cast<uint4*>(S.w1);
        for (uint32_t i = tid; i < MLP_H * MLP_IN / 8; i += INF_THREADS) d1[i] = s1[i];
        const uint4* s2 = reinterpret_cast<const uint4*>(W.w2);
        uint4* d2 = reinterpret_cast<uint4*>(S.w2);
        for (uint32_t i = tid; i < MLP_H * MLP_H / 8; i += INF_THREADS) d2[i] = s2[i];
        const uint4* s3 = reinterpret_cast<const uint4*>(W.w3);
        uint4* d3 = reinterpret_cast<uint4*>(S.w3);
        for (uint32_t i = tid; i < MLP_OUT * MLP_H / 8; i += INF_THREADS) d3[i] = s3[i];
        for (uint32_t i = tid; i < MLP_H; i += INF_THREADS) {
            S.b1[i] = W.b1[i];
            S.b2[i] = W.b2[i];
        }
        if (tid < MLP_OUT) S.b3[tid] = W.b3[tid];
    }
    if (tid < INF_GROUPS) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.mbar[tid])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.tbar[tid])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (tid == 0)
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&feat_map)) : "memory");
    if (warp == 0) {  // one warp allocates the tensor memory of the CTA
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_u32(&S.tmem_base)),
                     "r"((uint32_t)INF_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t mbar = smem_u32(&S.mbar[g]);
    const uint32_t tbar = smem_u32(&S.tbar[g]);
    const uint32_t tmem = S.tmem_base + g * 128u;        // this group's 128 columns
    bf16* act = S.act[g];
    bf16* planes = S.feat[g];
    const uint32_t quad = gwarp & 3u, half = gwarp >> 2;
    const uint32_t lane_addr = tmem + ((quad * 32u) << 16);  // this warp's TMEM lanes
    const uint32_t row = quad * 32u + (gtid & 31u);          // tile row = this thread's particle
    uint32_t phase = 0;
    bool ok = true;

    const uint32_t ntiles = (n + 127) / 128;
    const uint32_t first = blockIdx.x * INF_GROUPS + g, tstride = gridDim.x * INF_GROUPS;
    // tpend: 0, or 1 + the parity of a feature tile in flight whose arrival is not yet observed
    uint32_t tphase = 0, tpend = 0;
    if (first < ntiles) {
        if (gtid == 0) feat_tile_tma(planes, &feat_map, first * 128u, tbar);
        tpend = 1u + tphase;
    }
    for (uint32_t tile = first; tile < ntiles; tile += tstride) {
        const uint32_t p = tile * 128u + row;
        const bool live = p < n;
        // the tile's features (rows past the matrix are zeros; rows past n are computed and
        // not stored)
        ok = group_and(g, mbar_wait(tbar, tphase, spin_limit));
        tphase ^= 1u;
        if (!ok) break;
        tpend = 0;
        // the output step's reads of this particle, towards L2 while the three layers run
        if (half == 0 && live) {
            asm volatile("prefetch.global.L2 [%0];\n" ::"l"(conc_in + (size_t)p * NTF));
            if (genes) asm volatile("prefetch.global.L2 [%0];\n" ::"l"(genes + p));
        }
        tc_fence_after();
        if (gtid == 0 && !withhold) {
            issue_layer1(tmem, planes, S.w1);
            mma_commit(mbar);
        }
        ok = group_and(g, mbar_wait(mbar, phase, spin_limit));
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
        // layer 1 has read the planes: the next tile's features load under this tile's work
        if (tile + tstride < ntiles) {
            if (gtid == 0) feat_tile_tma(planes, &feat_map, (tile + tstride) * 128u, tbar);
            tpend = 1u + tphase;
        }
        // layer-1 epilogue: bias + GELU -> layer-2 operand (layer 1 has finished with `act`)
#pragma unroll
        for (uint32_t c0 = half * INF_COLS; c0 < (half + 1) * INF_COLS; c0 += 32) {
            float v[32];
            tmem_ld32(lane_addr + c0, v);
#pragma unroll
            for (int q = 0; q < 32; q += 8) {
                float h[8];
                bias_gelu8(v + q, S.b1 + c0 + q, h);
                put8(act, row, c0 + q, MLP_H, h);
            }
        }
        // the accumulator columns are read: layer 2 may overwrite them
        fence_async_smem();
        tc_fence_before();
        group_sync(g);
        tc_fence_after();
        if (gtid == 0 && !withhold) {
            issue_layer(tmem, act, S.w2, MLP_H, MLP_H);
            mma_commit(mbar);
        }
        ok = group_and(g, mbar_wait(mbar, phase, spin_limit));
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
        // layer-2 epilogue -> layer-3 operand (layer 2 has finished reading `act`)
#pragma unroll
        for (uint32_t c0 = half * INF_COLS; c0 < (half + 1) * INF_COLS; c0 += 32) {
            float v[32];
            tmem_ld32(lane_addr + c0, v);
#pragma unroll
            for (int q = 0; q < 32; q += 8) {
                float h[8];
                bias_gelu8(v + q, S.b2 + c0 + q, h);
                put8(act, row, c0 + q, MLP_H, h);
            }
        }
        fence_async_smem();
        tc_fence_before();
        group_sync(g);
        tc_fence_after();
        if (gtid == 0 && !withhold) {
            issue_layer(tmem, act, S.w3, MLP_H, MLP_OUT);
            mma_commit(mbar);
        }
        ok = group_and(g, mbar_wait(mbar, phase, spin_limit));
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
        if (half == 0) {
            float d[16];
            tmem_ld16(lane_addr + 0, d);
            if (live) {
                const float4* ci = reinterpret_cast<const float4*>(conc_in + (size_t)p * NTF);
                const float sc = feat_scale ? feat_scale[p] : 1.f;  // inputs' per-particle scale
                float c[16];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float4 x = ci[k];
                    c[4 * k] = x.x + sc * (d[4 * k] + S.b3[4 * k]);
                    c[4 * k + 1] = x.y + sc * (d[4 * k + 1] + S.b3[4 * k + 1]);
                    c[4 * k + 2] = x.z + sc * (d[4 * k + 2] + S.b3[4 * k + 2]);
                    c[4 * k + 3] = x.w + sc * (d[4 * k + 3] + S.b3[4 * k + 3]);
                }
                if (genes) {
                    const uint32_t gw = genes[p];
                    const bool judged = judge_step && (p % judge_stride) == judge_phase;
                    const bool fallback = (gw >> 31) & 1u;
                    if (judged || fallback) {
                        const float4* cp = reinterpret_cast<const float4*>(conc_plain + (size_t)p * NTF);
                        float pl[16];
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const float4 x = cp[k];
                            pl[4 * k] = x.x; pl[4 * k + 1] = x.y; pl[4 * k + 2] = x.z; pl[4 * k + 3] = x.w;
                        }
                        bool take = fallback;
                        if (judged && !fallback) {
                            // relative error of the particle: largest deviation over the
                            // largest plain concentration
                            float dev = 0.f, mag = 0.f;
#pragma unroll
                            for (int t = 0; t < 16; t++) {
                                dev = fmaxf(dev, fabsf(c[t] - pl[t]));
                                mag = fmaxf(mag, fabsf(pl[t]));
                            }
                            const float worst = dev / fmaxf(mag, 1e-30f);
                            atomicAdd(&stats[0], 1u);
                            atomicMax(&stats[2], __float_as_uint(worst));
                            if (!(worst <= threshold)) {  // hand the particle to the plain method
                                genes[p] = gw | 0x80000000u;
                                atomicAdd(&stats[1], 1u);
                                take = true;
                            }
                        }
                        if (take) {
#pragma unroll
                            for (int t = 0; t < 16; t++) c[t] = pl[t];
                        }
                    }
                }
                float4* co = reinterpret_cast<float4*>(conc_out + (size_t)p * NTF);
#pragma unroll
                for (int k = 0; k < 4; k++) co[k] = make_float4(c[4 * k], c[4 * k + 1], c[4 * k + 2], c[4 * k + 3]);
            }
        }
        // the output columns are read before the next tile's layer 1 overwrites them
        tc_fence_before();
        group_sync(g);
        tc_fence_after();
    }
    if (!ok) {
        // a wait gave up: record it and give the group's MMAs and feature load in flight one
        // more bounded wait each before the tensor memory and the CTA's shared memory go
        if (gtid == 0) {
            atomicOr(err, MLP_ERR_MBAR_TIMEOUT);
            mbar_wait(mbar, phase ^ 1u, spin_limit);
            if (tpend) mbar_wait(tbar, tpend - 1u, spin_limit);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(S.tmem_base),
                     "r"((uint32_t)INF_TMEM_COLS)
                     : "memory");
}

}  // namespace mg

// =============================================================================================
// Host side: parameters, training loop, normalisation, inference weights
// =============================================================================================
namespace mg {

namespace {

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

inline uint32_t blocks(size_t n, int t = 256) { return (uint32_t)((n + t - 1) / t); }

#define MLP_TRY(x)                             \
    do {                                       \
        cudaError_t e_ = (x);                  \
        if (e_ != cudaSuccess) return e_;      \
    } while (0)

}  // namespace

cudaError_t mlp_init_attributes() {
    MLP_TRY(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(GemmSmem)));
    return cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(InferSmem));
}

cudaError_t mlp_alloc(Mlp* m, uint64_t seed, cudaStream_t st) {
    std::memset(m, 0, sizeof(*m));
    m->st = st;
    MLP_TRY(cudaMalloc(&m->params, 4ull * P_COUNT * 4));
    m->grads = m->params + P_COUNT;
    m->adam_m = m->grads + P_COUNT;
    m->adam_v = m->adam_m + P_COUNT;
    MLP_TRY(cudaMalloc(&m->wb, sizeof(bf16) * P_COUNT));
    MLP_TRY(cudaMalloc(&m->norm, sizeof(float) * NORM_COUNT));
    MLP_TRY(cudaMalloc(&m->err, sizeof(uint32_t)));
    MLP_TRY(cudaMemsetAsync(m->err, 0, sizeof(uint32_t), st));
    const size_t inf_bytes = sizeof(bf16) * (MLP_H * MLP_IN + MLP_H * MLP_H + MLP_OUT * MLP_H) +
                             sizeof(float) * (2 * MLP_H + MLP_OUT);
    MLP_TRY(cudaMalloc(&m->inf_mem, inf_bytes));
    char* b = (char*)m->inf_mem;
    m->inf.w1 = (bf16*)b; b += sizeof(bf16) * MLP_H * MLP_IN;
    m->inf.w2 = (bf16*)b; b += sizeof(bf16) * MLP_H * MLP_H;
    m->inf.w3 = (bf16*)b; b += sizeof(bf16) * MLP_OUT * MLP_H;
    m->inf.b1 = (float*)b; b += sizeof(float) * MLP_H;
    m->inf.b2 = (float*)b; b += sizeof(float) * MLP_H;
    m->inf.b3 = (float*)b;
    // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases
    std::vector<float> p(P_COUNT, 0.f);
    uint64_t s = seed * 0x632be59bd9b4e019ull + 12345;
    auto fill = [&](int off, int rows, int cols, float gain) {
        const float a = gain / std::sqrt((float)cols);
        for (int i = 0; i < rows * cols; i++) {
            const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
            p[off + i] = (float)((2.0 * u - 1.0) * a);
        }
    };
    fill(P_W1, MLP_H, MLP_IN, 1.f);
    fill(P_W2, MLP_H, MLP_H, 1.f);
    fill(P_W3, MLP_OUT, MLP_H, 0.1f);
    std::vector<float> nrm(NORM_COUNT, 0.f);
    for (int i = 0; i < MLP_IN; i++) nrm[MLP_IN + i] = 1.f;            // isd_x
    for (int o = 0; o < MLP_OUT; o++) nrm[2 * MLP_IN + MLP_OUT + o] = 1.f;  // isd_y
    MLP_TRY(mlp_set_params(m, p.data()));
    MLP_TRY(cudaMemcpyAsync(m->norm, nrm.data(), sizeof(float) * NORM_COUNT, cudaMemcpyHostToDevice, st));
    MLP_TRY(cudaMemsetAsync(m->adam_m, 0, 2ull * P_COUNT * 4, st));
    m->adam_t = 0;
    return mlp_refresh_inference(m);
}

void mlp_free(Mlp* m) {
    cudaFree(m->params);
    cudaFree(m->wb);
    cudaFree(m->norm);
    cudaFree(m->err);
    cudaFree(m->inf_mem);
    cudaFree(m->ws);
    std::memset(m, 0, sizeof(*m));
}

cudaError_t mlp_set_params(Mlp* m, const float* host) {
    MLP_TRY(cudaMemcpyAsync(m->params, host, 4ull * P_COUNT, cudaMemcpyHostToDevice, m->st));
    k_to_bf16<<<blocks(P_COUNT), 256, 0, m->st>>>(m->params, m->wb, P_COUNT);
    return cudaGetLastError();
}

cudaError_t mlp_get_params(Mlp* m, float* host) {
    MLP_TRY(cudaMemcpyAsync(host, m->params, 4ull * P_COUNT, cudaMemcpyDeviceToHost, m->st));
    return cudaStreamSynchronize(m->st);
}

cudaError_t mlp_set_norm(Mlp* m, const float* host) {
    MLP_TRY(cudaMemcpyAsync(m->norm, host, sizeof(float) * NORM_COUNT, cudaMemcpyHostToDevice, m->st));
    return cudaStreamSynchronize(m->st);
}

cudaError_t mlp_get_norm(Mlp* m, float* host) {
    MLP_TRY(cudaMemcpyAsync(host, m->norm, sizeof(float) * NORM_COUNT, cudaMemcpyDeviceToHost, m->st));
    return cudaStreamSynchronize(m->st);
}

// Inference weights: input normalisation folded into layer 1, output scaling into layer 3,
// matrices re-laid out as tcgen05 K-major core matrices.
cudaError_t mlp_refresh_inference(Mlp* m) {
    std::vector<float> p(P_COUNT), nrm(NORM_COUNT);
    MLP_TRY(mlp_get_params(m, p.data()));
    MLP_TRY(mlp_get_norm(m, nrm.data()));
    const float* mx = nrm.data();
    const float* sx = mx + MLP_IN;
    const float* my = sx + MLP_IN;
    const float* sy = my + MLP_OUT;
    std::vector<bf16> w1(MLP_H * MLP_IN), w2(MLP_H * MLP_H), w3(MLP_OUT * MLP_H);
    std::vector<float> b1(MLP_H), b2(MLP_H), b3(MLP_OUT);
    for (int o = 0; o < MLP_H; o++) {
        double bias = p[P_B1 + o];
        for (int i = 0; i < MLP_IN; i++) {
            const float w = p[P_W1 + o * MLP_IN + i] * sx[i];
            w1[core_offset(o, i, MLP_IN)] = __float2bfloat16(w);
            bias -= (double)w * mx[i];
        }
        b1[o] = (float)bias;
        b2[o] = p[P_B2 + o];
        for (int j = 0; j < MLP_H; j++) w2[core_offset(o, j, MLP_H)] = __float2bfloat16(p[P_W2 + o * MLP_H + j]);
    }
    for (int o = 0; o < MLP_OUT; o++) {
        const float inv = 1.f / sy[o];
        for (int j = 0; j < MLP_H; j++)
            w3[core_offset(o, j, MLP_H)] = __float2bfloat16(p[P_W3 + o * MLP_H + j] * inv);
        b3[o] = p[P_B3 + o] * inv + my[o];
    }
    MLP_TRY(cudaMemcpyAsync(m->inf.w1, w1.data(), sizeof(bf16) * w1.size(), cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemcpyAsync(m->inf.w2, w2.data(), sizeof(bf16) * w2.size(), cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemcpyAsync(m->inf.w3, w3.data(), sizeof(bf16) * w3.size(), cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemcpyAsync(m->inf.b1, b1.data(), sizeof(float) * MLP_H, cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemcpyAsync(m->inf.b2, b2.data(), sizeof(float) * MLP_H, cudaMemcpyHostToDevice, m->st));
    MLP_TRY(cudaMemcpyAsync(m->inf.b3, b3.data(), sizeof(float) * MLP_OUT, cudaMemcpyHostToDevice, m->st));
    return cudaStreamSynchronize(m->st);
}

// Per-column mean and inverse standard deviation of the dataset (constant columns get 1).
cudaError_t mlp_fit_norm(Mlp* m, const float* dx, const float* dy, uint64_t rows) {
    double* acc = nullptr;
    MLP_TRY(cudaMalloc(&acc, sizeof(double) * 2 * (MLP_IN + MLP_OUT)));
    MLP_TRY(cudaMemsetAsync(acc, 0, sizeof(double) * 2 * (MLP_IN + MLP_OUT), m->st));
    k_col_stats<<<dim3(256, MLP_IN), 256, 0, m->st>>>(dx, rows, MLP_IN, acc);
    k_col_stats<<<dim3(256, MLP_OUT), 256, 0, m->st>>>(dy, rows, MLP_OUT, acc + 2 * MLP_IN);
    std::vector<double> h(2 * (MLP_IN + MLP_OUT));
    cudaError_t e = cudaMemcpyAsync(h.data(), acc, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
    cudaFree(acc);
    if (e != cudaSuccess) return e;
    std::vector<float> nrm(NORM_COUNT);
    auto put = [&](int col, int mu_at, int isd_at, const double* a) {
        const double mean = a[0] / (double)rows;
        const double var = a[1] / (double)rows - mean * mean;
        const double sd = var > 1e-20 ? std::sqrt(var) : 0.0;
        nrm[mu_at] = (float)mean;
        nrm[isd_at] = sd > 0.0 ? (float)(1.0 / sd) : 1.f;
        (void)col;
    };
    for (int i = 0; i < MLP_IN; i++) put(i, i, MLP_IN + i, &h[2 * i]);
    for (int o = 0; o < MLP_OUT; o++) put(o, 2 * MLP_IN + o, 2 * MLP_IN + MLP_OUT + o, &h[2 * (MLP_IN + o)]);
    return mlp_set_norm(m, nrm.data());
}

namespace {

// The training GEMMs' error bits: a completion wait that gave up reads as cudaErrorTimeout.
cudaError_t check_err(Mlp* m) {
    uint32_t bits = 0;
    MLP_TRY(cudaMemcpyAsync(&bits, m->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    return bits ? cudaErrorTimeout : cudaSuccess;
}

struct Workspace {
    bf16 *X, *H1, *H2, *dY16, *dZ16;
    float *Y, *Z1, *Z2, *Z3, *dY32, *dH, *dZ32;
    double* loss;
};

cudaError_t workspace(Mlp* m, uint32_t B, Workspace* w) {
    const size_t need = (size_t)B * (2 * MLP_IN + 2 * MLP_H * 3 + 2 * MLP_OUT) +  // bf16 arrays
                        (size_t)B * 4 * (MLP_OUT * 3 + MLP_H * 4) + 64;
    if (m->ws_batch < B) {
        cudaFree(m->ws);
        m->ws = nullptr;
        m->ws_batch = 0;
        MLP_TRY(cudaMalloc(&m->ws, need + 4096));
        m->ws_batch = B;
    }
    char* p = (char*)m->ws;
    auto take = [&](size_t bytes) { char* r = p; p += (bytes + 255) & ~(size_t)255; return r; };
    w->loss = (double*)take(64);
    w->X = (bf16*)take(2ull * B * MLP_IN);
    w->H1 = (bf16*)take(2ull * B * MLP_H);
    w->H2 = (bf16*)take(2ull * B * MLP_H);
    w->dZ16 = (bf16*)take(2ull * B * MLP_H);
    w->dY16 = (bf16*)take(2ull * B * MLP_OUT);
    w->Y = (float*)take(4ull * B * MLP_OUT);
    w->Z3 = (float*)take(4ull * B * MLP_OUT);
    w->dY32 = (float*)take(4ull * B * MLP_OUT);
    w->Z1 = (float*)take(4ull * B * MLP_H);
    w->Z2 = (float*)take(4ull * B * MLP_H);
    w->dH = (float*)take(4ull * B * MLP_H);
    w->dZ32 = (float*)take(4ull * B * MLP_H);
    return cudaSuccess;
}

// Forward and backward of one batch already in w->X / w->Y; gradients into m->grads.
void fwd_bwd(Mlp* m, const Workspace& w, uint32_t B) {
    cudaStream_t st = m->st;
    const bf16* W1 = m->wb + P_W1;
    const bf16* W2 = m->wb + P_W2;
    const bf16* W3 = m->wb + P_W3;
    // weight gradients reduce over the batch: split K into ranges of at least 512 rows
    const int split = (int)std::max<uint32_t>(1u, std::min<uint32_t>(128u, B / 512u));
    launch_gemm_bf16(B, MLP_H, MLP_IN, w.X, MLP_IN, 1, W1, 1, MLP_IN, w.Z1, MLP_H, 1, m->err, st);
    k_bias_act<<<blocks((size_t)B * MLP_H), 256, 0, st>>>(w.Z1, m->params + P_B1, MLP_H, (size_t)B * MLP_H, w.H1);
    launch_gemm_bf16(B, MLP_H, MLP_H, w.H1, MLP_H, 1, W2, 1, MLP_H, w.Z2, MLP_H, 1, m->err, st);
    k_bias_act<<<blocks((size_t)B * MLP_H), 256, 0, st>>>(w.Z2, m->params + P_B2, MLP_H, (size_t)B * MLP_H, w.H2);
    launch_gemm_bf16(B, MLP_OUT, MLP_H, w.H2, MLP_H, 1, W3, 1, MLP_H, w.Z3, MLP_OUT, 1, m->err, st);
    k_bias_act<<<blocks((size_t)B * MLP_OUT), 256, 0, st>>>(w.Z3, m->params + P_B3, MLP_OUT, (size_t)B * MLP_OUT, nullptr);
    cudaMemsetAsync(w.loss, 0, sizeof(double), st);
    k_out_grad<<<blocks((size_t)B * MLP_OUT), 256, 0, st>>>(w.Z3, w.Y, (size_t)B * MLP_OUT,
                                                          1.f / ((float)B * MLP_OUT), w.dY16, w.dY32, w.loss);
    cudaMemsetAsync(m->grads, 0, 4ull * P_COUNT, st);
    // layer 3
    launch_gemm_bf16(MLP_OUT, MLP_H, B, w.dY16, 1, MLP_OUT, w.H2, MLP_H, 1, m->grads + P_W3, MLP_H, split, m->err, st);
    k_colsum<<<MLP_OUT, 256, 0, st>>>(w.dY32, B, MLP_OUT, m->grads + P_B3);
    launch_gemm_bf16(B, MLP_H, MLP_OUT, w.dY16, MLP_OUT, 1, W3, MLP_H, 1, w.dH, MLP_H, 1, m->err, st);
    k_act_grad<<<blocks((size_t)B * MLP_H), 256, 0, st>>>(w.dH, w.Z2, (size_t)B * MLP_H, w.dZ16, w.dZ32);
    // layer 2
    launch_gemm_bf16(MLP_H, MLP_H, B, w.dZ16, 1, MLP_H, w.H1, MLP_H, 1, m->grads + P_W2, MLP_H, split, m->err, st);
    k_colsum<<<MLP_H, 256, 0, st>>>(w.dZ32, B, MLP_H, m->grads + P_B2);
    launch_gemm_bf16(B, MLP_H, MLP_H, w.dZ16, MLP_H, 1, W2, MLP_H, 1, w.dH, MLP_H, 1, m->err, st);
    k_act_grad<<<blocks((size_t)B * MLP_H), 256, 0, st>>>(w.dH, w.Z1, (size_t)B * MLP_H, w.dZ16, w.dZ32);
    // layer 1
    launch_gemm_bf16(MLP_H, MLP_IN, B, w.dZ16, 1, MLP_H, w.X, MLP_IN, 1, m->grads + P_W1, MLP_IN, split, m->err, st);
    k_colsum<<<MLP_H, 256, 0, st>>>(w.dZ32, B, MLP_H, m->grads + P_B1);
}

}  // namespace

cudaError_t mlp_train(Mlp* m, const float* dx, const float* dy, uint64_t rows, uint32_t steps,
                      uint32_t B, float lr, uint64_t seed, float* loss_host) {
    if (rows == 0 || B == 0) return cudaErrorInvalidValue;
    Workspace w;
    MLP_TRY(workspace(m, B, &w));
    MLP_TRY(cudaMemsetAsync(m->err, 0, sizeof(uint32_t), m->st));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (uint32_t s = 0; s < steps; s++) {
        k_make_batch<<<blocks(B), 256, 0, m->st>>>(dx, dy, rows, B, mix_seed(seed, m->adam_t), m->norm,
                                                   w.X, w.Y, 0);
        fwd_bwd(m, w, B);
        m->adam_t++;
        const float c1 = 1.f - std::pow(b1, (float)m->adam_t);
        const float c2 = 1.f - std::pow(b2, (float)m->adam_t);
        k_adam<<<blocks(P_COUNT), 256, 0, m->st>>>(m->params, m->grads, m->adam_m, m->adam_v, P_COUNT, lr,
                                                   b1, b2, eps, c1, c2);
        k_to_bf16<<<blocks(P_COUNT), 256, 0, m->st>>>(m->params, m->wb, P_COUNT);
        if (loss_host) {
            double l = 0;
            MLP_TRY(cudaMemcpyAsync(&l, w.loss, sizeof(double), cudaMemcpyDeviceToHost, m->st));
            MLP_TRY(cudaStreamSynchronize(m->st));
            loss_host[s] = (float)(l / ((double)B * MLP_OUT));
        }
    }
    MLP_TRY(cudaGetLastError());
    MLP_TRY(check_err(m));
    return mlp_refresh_inference(m);
}

cudaError_t mlp_grad(Mlp* m, const float* dx, const float* dy, uint32_t n, float* grads_host,
                     double* loss) {
    Workspace w;
    MLP_TRY(workspace(m, n, &w));
    MLP_TRY(cudaMemsetAsync(m->err, 0, sizeof(uint32_t), m->st));
    k_make_batch<<<blocks(n), 256, 0, m->st>>>(dx, dy, n, n, 0, m->norm, w.X, w.Y, 1);
    fwd_bwd(m, w, n);
    MLP_TRY(cudaGetLastError());
    MLP_TRY(check_err(m));
    MLP_TRY(cudaMemcpyAsync(grads_host, m->grads, 4ull * P_COUNT, cudaMemcpyDeviceToHost, m->st));
    double l = 0;
    MLP_TRY(cudaMemcpyAsync(&l, w.loss, sizeof(double), cudaMemcpyDeviceToHost, m->st));
    MLP_TRY(cudaStreamSynchronize(m->st));
    if (loss) *loss = l / ((double)n * MLP_OUT);
    return cudaSuccess;
}

// cuTensorMapEncodeTiled, looked up once through the runtime (no link against the driver
// library).
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

cudaError_t make_feat_map(const bf16* feat, uint32_t rows, CUtensorMap* map) {
    // looked up once (a function-local static: initialised by one thread, seen by all)
    static const EncodeTiled encode = []() -> EncodeTiled {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<EncodeTiled>(fn);
    }();
    if (!encode) return cudaErrorNotSupported;
    // a 16-byte aligned base, a 96-byte row stride and 16-byte boxes along the features
    if ((reinterpret_cast<uintptr_t>(feat) & 15u) != 0 || rows == 0) return cudaErrorInvalidValue;
    const cuuint64_t dims[2] = {(cuuint64_t)MLP_IN, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)MLP_IN * sizeof(bf16)};
    const cuuint32_t box[2] = {8u, 128u};
    const cuuint32_t estride[2] = {1u, 1u};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(feat), dims, strides,
                              box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

void launch_mlp_infer(const Mlp* m, const CUtensorMap& feat_map, const float* feat_scale, const float* conc_in,
                      const float* conc_plain,
                      float* conc_out, uint32_t* genes, const uint32_t* nactive, uint32_t n_override,
                      const uint32_t* step, uint32_t period, uint32_t stride, float threshold,
                      uint32_t* stats, uint32_t* err, int num_sms, cudaStream_t st) {
    k_mlp_infer<<<num_sms, INF_THREADS, sizeof(InferSmem), st>>>(
        m->inf, feat_map, feat_scale, conc_in, conc_plain, conc_out, genes, nactive, n_override, step,
        period, stride,
        threshold, stats, err, MBAR_SPIN_LIMIT, 0u);
}

// Failure-detection self-test of the tensor-core completion wait: one inference CTA over one
// tile whose MMAs are withheld, so its mbarrier is never arrived on and the wait runs out
// after spin_limit polls; the CTA then records MLP_ERR_MBAR_TIMEOUT, frees its tensor memory
// and returns.  Returns the kernel's error bits; everything it touches is its own.
cudaError_t mlp_selftest_wait_timeout(uint32_t spin_limit, uint32_t* err_bits, cudaStream_t st) {
    Mlp m;
    std::memset(&m, 0, sizeof(m));
    cudaError_t e = mlp_init_attributes();
    if (e == cudaSuccess) e = mlp_alloc(&m, 1, st);
    bf16* feat = nullptr;
    float* conc = nullptr;
    uint32_t* err = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&feat, sizeof(bf16) * 128 * MLP_IN);
    if (e == cudaSuccess) e = cudaMalloc(&conc, sizeof(float) * 2 * 128 * NTF);
    if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(feat, 0, sizeof(bf16) * 128 * MLP_IN, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(conc, 0, sizeof(float) * 2 * 128 * NTF, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    CUtensorMap map;
    if (e == cudaSuccess) e = make_feat_map(feat, 128, &map);
    if (e == cudaSuccess) {
        k_mlp_infer<<<1, INF_THREADS, sizeof(InferSmem), st>>>(
            m.inf, map, nullptr, conc, nullptr, conc + 128 * NTF, nullptr, nullptr, 128u, nullptr,
            0u, 0u, 0.f, nullptr, err, spin_limit, 1u);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(err_bits, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(feat);
    cudaFree(conc);
    cudaFree(err);
    mlp_free(&m);
    return e;
}

// Failure-detection self-test of the training GEMM's completion waits: one CTA of a 128 x 16 x
// 192 product whose MMAs are withheld, so the wait for the first chunk's buffer runs out after
// spin_limit polls; the CTA records MLP_ERR_MBAR_TIMEOUT, frees its tensor memory and returns.
cudaError_t mlp_selftest_gemm_wait_timeout(uint32_t spin_limit, uint32_t* err_bits, cudaStream_t st) {
    const int M = 128, N = 16, K = 192;
    bf16 *a = nullptr, *b = nullptr;
    float* c = nullptr;
    uint32_t* err = nullptr;
    cudaError_t e = mlp_init_attributes();
    if (e == cudaSuccess) e = cudaMalloc(&a, sizeof(bf16) * M * K);
    if (e == cudaSuccess) e = cudaMalloc(&b, sizeof(bf16) * N * K);
    if (e == cudaSuccess) e = cudaMalloc(&c, sizeof(float) * M * N);
    if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(a, 0, sizeof(bf16) * M * K, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b, 0, sizeof(bf16) * N * K, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        const GemmOperand ga = gemm_operand(a, K, 1), gb = gemm_operand(b, K, 1);
        k_gemm_tc<<<dim3(1, 1, 1), TG_THREADS, sizeof(GemmSmem), st>>>(M, N, K, ga, gb, c, N, 1, 1, err,
                                                                       spin_limit, 1u);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(err_bits, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(a);
    cudaFree(b);
    cudaFree(c);
    cudaFree(err);
    return e;
}

}  // namespace mg
