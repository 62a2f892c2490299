// mg_sort.cu - grid binning, prefix sum and the stable counting sort (rows a2-a4).
//
// Reference: insertParticles (fluid_system_cuda.cu:53-100), prefixSum/prefixFixup
// (cuda:136-183, host_CUDA.cpp:307-407), countingSortFull (cuda:196-296).
//
// The reference assigns each particle its rank in a cell with atomicAdd, so the sorted order
// depends on the thread schedule.  Here the sorted order is the stable one (rank = number of
// earlier-index particles in the same cell, i.e. a serial execution of insertParticles):
//   insert   : cell of every particle, per-cell counts (warp-aggregated atomics) and an
//              arrival rank that is only used to scatter indices into their cell's segment;
//   scan     : single-pass exclusive scan with decoupled look-back (a warp reads 32
//              predecessor tiles per round) -> per-cell offsets;
//   place    : order[offset[cell] + arrival rank] = i, with the (sub-cell code, i) key;
//   cellsort : the stable rank of every particle in its cell (one thread per particle for
//              cells <= 256 particles; block tier <= 8192, ordered stream compaction above),
//              which yields sorted[] (sorted -> old) and newidx[] (old -> sorted), and the
//              density pass's processing order work[];
//   gather   : every carried field is gathered through sorted[]; the bond records stay at the
//              particles' origins, their partners and the incoming-bond owners are remapped
//              through newidx[] (in up to three kernels when parts of the state are still
//              being uploaded).
#include <cuda/atomic>
#include <cfloat>
#include "mg_internal.cuh"

#ifndef MG_SUB_ORDER
#define MG_SUB_ORDER 1  // in-cell processing order: 1 x-major slabs, 0 mirrored Morton
#endif

namespace mg {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Cell of a position (cuda:70-79): gcf = (pos - gridMin) * gridDelta truncated toward zero,
// valid when 1 <= gc <= gridScanMax on every axis.  Written as float range tests so that NaN
// and out-of-range values never go through a float->int conversion.
__device__ __forceinline__ uint32_t cell_of(const DevParams& P, float4 p) {
    float gx = (p.x - P.gmin[0]) * P.gdelta[0];
    float gy = (p.y - P.gmin[1]) * P.gdelta[1];
    float gz = (p.z - P.gmin[2]) * P.gdelta[2];
    if (!(gx >= 1.0f && gx < (float)(P.scanmax[0] + 1))) return UNDEF;
    if (!(gy >= 1.0f && gy < (float)(P.scanmax[1] + 1))) return UNDEF;
    if (!(gz >= 1.0f && gz < (float)(P.scanmax[2] + 1))) return UNDEF;
    int cx = (int)gx, cy = (int)gy, cz = (int)gz;
    return (uint32_t)((cy * P.res[2] + cz) * P.res[0] + cx);
}

// The same for a particle of a packed system: its instance's grid in its instance's frame,
// placed in the instance's slab of the shared grid (rows ybase ..).
__device__ __forceinline__ uint32_t cell_of(const DevParams& P, float4 p, const uint32_t* iid, uint32_t i) {
    if (!iid) return cell_of(P, p);
    const uint32_t k = iid[i];
    if (k >= (uint32_t)P.n_inst) return UNDEF;
    const InstParams& I = P.inst[k];
    float gx = (p.x - I.gmin[0]) * I.gdelta[0];
    float gy = (p.y - I.gmin[1]) * I.gdelta[1];
    float gz = (p.z - I.gmin[2]) * I.gdelta[2];
    if (!(gx >= 1.0f && gx < (float)(I.scanmax[0] + 1))) return UNDEF;
    if (!(gy >= 1.0f && gy < (float)(I.scanmax[1] + 1))) return UNDEF;
    if (!(gz >= 1.0f && gz < (float)(I.scanmax[2] + 1))) return UNDEF;
    int cx = (int)gx, cy = (int)gy + I.ybase, cz = (int)gz;
    return (uint32_t)((cy * P.res[2] + cz) * P.res[0] + cx);
}

// Morton code of the sub-cell holding a position inside its cell: 2^sub_bits sub-cells per axis
// (sub_bits 1 or 2) from the fractional part of the cell coordinate.  Only the density pass's
// processing order uses it, never a result.
// With `warp_order` (the order for the warp-cooperative searches), the code sorts x first: the
// cells are ordered along x, so a warp that takes the tail of one cell and the head of the next
// covers a thin slab on both sides of their shared face, and a warp inside one cell a slab as
// compact as a Morton half-cell (MG_SUB_ORDER 0 keeps Morton codes with the y and z
// coordinates mirrored in odd-x cells).  Without it, Morton codes (bit a = level-0 half of axis
// a, bit 3 + a = level-1), which the per-lane fine-cell search reads as positions.
__device__ __forceinline__ uint32_t sub_of(const DevParams& P, float4 p, bool warp_order,
                                           const InstParams* I = nullptr) {
    const float* gmin = I ? I->gmin : P.gmin;
    const float* gdelta = I ? I->gdelta : P.gdelta;
    const float g[3] = {(p.x - gmin[0]) * gdelta[0], (p.y - gmin[1]) * gdelta[1],
                        (p.z - gmin[2]) * gdelta[2]};
    const int nsub = 1 << P.sub_bits;
    int q[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int v = (int)((g[a] - floorf(g[a])) * (float)nsub);
        q[a] = v < 0 ? 0 : (v > nsub - 1 ? nsub - 1 : v);
    }
    if (warp_order && MG_SUB_ORDER == 1) return (uint32_t)((q[0] * nsub + q[1]) * nsub + q[2]);
    const bool flip = warp_order && (((int)floorf(g[0])) & 1);
    uint32_t code = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int qa = (flip && a > 0) ? nsub - 1 - q[a] : q[a];
        code |= ((uint32_t)(qa & 1) << a) | ((uint32_t)((qa >> 1) & 1) << (3 + a));
    }
    return P.sub_bits == 1 ? code & 7u : code;
}

// ---- insert -------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_insert(DevParams P, const float4* __restrict__ pos,
                                                uint32_t* __restrict__ cell,
                                                uint32_t* __restrict__ arank,
                                                uint32_t* __restrict__ newidx,
                                                uint32_t* __restrict__ count,
                                                uint8_t* __restrict__ sub,
                                                uint32_t* __restrict__ step, bool warp_order,
                                                const uint32_t* __restrict__ iid) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *step += 1u;  // step counter read by the later kernels of this step
    bool in = i < P.cap;
    uint32_t c = UNDEF;
    if (in) {
        const float4 pi = pos[i];
        c = cell_of(P, pi, iid, i);
        cell[i] = c;
        newidx[i] = UNDEF;  // overwritten by the cell sort for particles inside the window
        if (c != UNDEF) sub[i] = (uint8_t)sub_of(P, pi, warp_order, iid ? P.inst + iid[i] : nullptr);
    }
    bool valid = in && c != UNDEF;
    unsigned active = __ballot_sync(0xffffffffu, valid);
    if (valid) {
        unsigned peers = __match_any_sync(active, c);
        int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if ((int)lane_id() == leader) base = atomicAdd(&count[c], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        unsigned lt = (1u << lane_id()) - 1u;
        arank[i] = base + (uint32_t)__popc(peers & lt);
    }
}

// Zeroes the bin counts, the scan's tile status words and the sort's first two counters
// before the bin pass: one kernel instead of three memsets.
__global__ void __launch_bounds__(256) k_clear_bins(uint32_t* __restrict__ count, uint32_t cells,
                                                    unsigned long long* __restrict__ status,
                                                    uint32_t nstatus, uint32_t* __restrict__ counters) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const uint32_t n4 = cells / 4u;  // count is 256-byte aligned
    uint4* c4 = reinterpret_cast<uint4*>(count);
    for (uint32_t k = i; k < n4; k += stride) c4[k] = make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t k = n4 * 4u + i; k < cells; k += stride) count[k] = 0u;
    for (uint32_t k = i; k < nstatus; k += stride) status[k] = 0ull;
    if (i < 2u) counters[i] = 0u;
}

void launch_clear_bins(const DevParams& P, const Scratch& s, int num_sms, cudaStream_t st) {
    k_clear_bins<<<(uint32_t)num_sms * 4u, 256, 0, st>>>(s.count, P.cells, s.scan_status,
                                                        (uint32_t)scan_status_words(P.cells), s.counters);
}

void launch_insert(const DevParams& P, const Carried& cur, const Scratch& s, bool warp_order,
                   cudaStream_t st) {
    uint32_t blocks = (P.cap + 255) / 256;
    k_insert<<<blocks, 256, 0, st>>>(P, cur.pos, s.cell, s.arank, s.newidx, s.count, s.sub,
                                      s.counters + 5, warp_order, cur.iid);
}

// ---- single-pass scan (decoupled look-back) ------------------------------------------------
// Tile status word: high 32 bits = flag (0 not ready, 1 aggregate, 2 inclusive prefix),
// low 32 bits = value.  Flag and value are published by one 64-bit atomic store, so a relaxed
// load that sees the flag also sees its value.  Tiles take their index from a ticket counter,
// so every tile a block waits on has already started; each wait is still bounded and sets
// ERR_SCAN_TIMEOUT when it gives up.
size_t scan_status_words(uint32_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

template <int ITEMS>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan(const uint32_t* __restrict__ in,
                                                       uint32_t* __restrict__ out, uint32_t n,
                                                       unsigned long long* status,
                                                       uint32_t* ticket, uint32_t* total,
                                                       uint32_t* err, uint32_t spin_limit) {
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    constexpr uint32_t TILE = SCAN_THREADS * ITEMS;
    const uint32_t ntiles = (n + TILE - 1) / TILE;
    const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
    const uint32_t per_warp = TILE / (SCAN_THREADS / 32);
    const uint32_t wbase = tile * TILE + warp * per_warp;
    uint32_t vals[ITEMS];
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
        uint32_t idx = wbase + k * 32 + lane;
        uint32_t v = idx < n ? in[idx] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, x, d);
            if ((int)lane >= d) x += t;
        }
        vals[k] = run + x - v;
        run += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) s_warp[warp] = run;
    __syncthreads();
    if (warp == 0) {
        const int nw = SCAN_THREADS / 32;
        uint32_t w = (int)lane < nw ? s_warp[lane] : 0u;
        uint32_t incl = w;
#pragma unroll
        for (int d = 1; d < nw; d <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
            if ((int)lane >= d) incl += t;
        }
        uint32_t agg = __shfl_sync(0xffffffffu, incl, nw - 1);
        if ((int)lane < nw) s_warp[lane] = incl - w;
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> me(status[tile]);
        if (lane == 0) me.store(((tile == 0 ? 2ull : 1ull) << 32) | agg, cuda::memory_order_relaxed);
        // Look-back by the whole warp: lane i reads the status of tile (end - i), 32 tiles per
        // round.  A round completes when every tile from end down to the nearest one holding
        // an inclusive prefix has published; their values sum to this tile's exclusive prefix.
        uint32_t excl = 0;
        if (tile > 0) {
            int64_t end = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (true) {
                const int64_t t = end - (int64_t)lane;
                unsigned long long sw = 2ull << 32;  // before tile 0: an inclusive prefix of 0
                if (t >= 0) {
                    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> prev(status[t]);
                    sw = prev.load(cuda::memory_order_relaxed);
                }
                const uint32_t flag = (uint32_t)(sw >> 32);
                const unsigned inclusive = __ballot_sync(0xffffffffu, flag == 2);
                const unsigned unready = __ballot_sync(0xffffffffu, flag == 0);
                const int stop = inclusive ? __ffs(inclusive) - 1 : 31;  // last lane to sum
                const unsigned needed = stop == 31 ? 0xffffffffu : ((2u << stop) - 1u);
                if (unready & needed) {
                    if (++spins > spin_limit) {
                        if (lane == 0) atomicOr(err, ERR_SCAN_TIMEOUT);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                uint32_t v = (int)lane <= stop ? (uint32_t)sw : 0u;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
                excl += v;
                if (inclusive) break;
                end -= 32;
            }
            if (lane == 0) me.store((2ull << 32) | (uint32_t)(excl + agg), cuda::memory_order_relaxed);
        }
        if (lane == 0) {
            s_prefix = excl;
            if (tile == ntiles - 1 && total) *total = excl + agg;
        }
    }
    __syncthreads();
    const uint32_t pre = s_prefix + s_warp[warp];
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
        uint32_t idx = wbase + k * 32 + lane;
        if (idx < n) out[idx] = pre + vals[k];
    }
}

void launch_scan(const uint32_t* in, uint32_t* out, uint32_t n, unsigned long long* status,
                 uint32_t* ticket, uint32_t* total, uint32_t* err, cudaStream_t st, bool narrow) {
    if (n == 0) return;
    if (narrow) {
        const uint32_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
        k_scan<SCAN_ITEMS><<<tiles, SCAN_THREADS, 0, st>>>(in, out, n, status, ticket, total, err, SPIN_LIMIT);
    } else {
        constexpr uint32_t WIDE_TILE = SCAN_THREADS * WIDE_SCAN_ITEMS;
        const uint32_t tiles = (n + WIDE_TILE - 1) / WIDE_TILE;
        k_scan<WIDE_SCAN_ITEMS><<<tiles, SCAN_THREADS, 0, st>>>(in, out, n, status, ticket, total, err,
                                                                 SPIN_LIMIT);
    }
}

// Failure-detection self-test of the look-back wait: a scan of 8 tiles whose first tile is
// never launched (the ticket starts at 1 and 7 blocks run), so its status word stays
// unpublished and every other tile's wait runs out after spin_limit polls.  Returns the
// kernel's error bits (ERR_SCAN_TIMEOUT expected); everything it touches is its own.
cudaError_t scan_selftest_wait_timeout(uint32_t spin_limit, uint32_t* err_bits, cudaStream_t st) {
    const uint32_t tiles = 8, n = tiles * SCAN_TILE;
    uint32_t *counts = nullptr, *offsets = nullptr, *words = nullptr;
    unsigned long long* status = nullptr;
    cudaError_t e = cudaMalloc(&counts, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&offsets, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&status, sizeof(unsigned long long) * tiles);
    if (e == cudaSuccess) e = cudaMalloc(&words, sizeof(uint32_t) * 2);  // ticket, error
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(unsigned long long) * tiles, st);
    const uint32_t init[2] = {1u, 0u};
    if (e == cudaSuccess) e = cudaMemcpyAsync(words, init, sizeof init, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_scan<SCAN_ITEMS><<<tiles - 1, SCAN_THREADS, 0, st>>>(counts, offsets, n, status, words, nullptr,
                                                   words + 1, spin_limit);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(err_bits, words + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(counts);
    cudaFree(offsets);
    cudaFree(status);
    cudaFree(words);
    return e;
}

// ---- place ----------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_place(uint32_t cap, const uint32_t* __restrict__ cell,
                                               const uint32_t* __restrict__ arank,
                                               const uint32_t* __restrict__ offset,
                                               const uint8_t* __restrict__ sub,
                                               uint32_t* __restrict__ order,
                                               unsigned long long* __restrict__ okey) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    uint32_t c = cell[i];
    if (c == UNDEF) return;
    const uint32_t slot = offset[c] + arank[i];
    order[slot] = i;
    okey[slot] = ((unsigned long long)sub[i] << 32) | i;
}

void launch_place(const DevParams& P, const Scratch& s, cudaStream_t st) {
    uint32_t blocks = (P.cap + 255) / 256;
    k_place<<<blocks, 256, 0, st>>>(P.cap, s.cell, s.arank, s.offset, s.sub, s.order, s.okey);
}

// ---- cell sort ------------------------------------------------------------------------------
// One thread per arrival slot s < nactive: particle x = order[s] of cell c counts the members
// of c with a smaller index (its stable rank r) and the members whose (sub-cell code, index)
// key is smaller (its rank w in the processing order), one 64-bit key per member.  Members are
// read in the same order by every lane of a warp that shares the cell, so the loads broadcast.  Cells above
// WARP_CELL_MAX particles go to the block tier through the big-cell list.
__global__ void __launch_bounds__(256) k_cellsort(const uint32_t* __restrict__ cell,
                                                  const uint32_t* __restrict__ count,
                                                  const uint32_t* __restrict__ offset,
                                                  const unsigned long long* __restrict__ okey,
                                                  uint32_t* __restrict__ sorted,
                                                  uint32_t* __restrict__ newidx,
                                                  uint32_t* __restrict__ work,
                                                  unsigned long long* __restrict__ subcnt,
                                                  uint32_t* __restrict__ big_list,
                                                  uint32_t* __restrict__ big_count,
                                                  uint32_t* __restrict__ err,
                                                  const uint32_t* __restrict__ nactive_p) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= *nactive_p) return;
    const unsigned long long kx = okey[s];
    const uint32_t x = (uint32_t)kx;
    const uint32_t c = cell[x];
    const uint32_t off = offset[c], n = count[c];
    if (n > (uint32_t)WARP_CELL_MAX) {
        if (s == off) {
            const uint32_t k = atomicAdd(big_count, 1u);
            if (k < BIG_LIST_CAP) big_list[k] = c;
            else atomicOr(err, ERR_BIG_LIST_OVERFLOW);
        }
        return;
    }
    uint32_t r = 0, w = 0;
#pragma unroll 4
    for (uint32_t m = 0; m < n; m++) {
        const unsigned long long km = __ldg(okey + off + m);
        r += (uint32_t)km < x ? 1u : 0u;
        w += km < kx ? 1u : 0u;
    }
    sorted[off + r] = x;
    newidx[x] = off + r;
    work[off + w] = off + r;
    // per sub-cell code counts, 8 bits each (with 2x2x2 sub-cells the codes are 0..7; the
    // table was zeroed before this pass)
    if (subcnt && n < (uint32_t)WARP_CELL_MAX) atomicAdd(subcnt + c, 1ull << (8 * ((uint32_t)(kx >> 32) & 7u)));
}

constexpr int BIG_THREADS = 512;

__global__ void __launch_bounds__(BIG_THREADS) k_cellsort_big(uint32_t cap,
                                                              const uint32_t* __restrict__ cell,
                                                              const uint32_t* __restrict__ count,
                                                              const uint32_t* __restrict__ offset,
                                                              const uint32_t* __restrict__ order,
                                                              uint32_t* __restrict__ sorted,
                                                              uint32_t* __restrict__ newidx,
                                                              uint32_t* __restrict__ work,
                                                              const uint32_t* __restrict__ big_list,
                                                              const uint32_t* __restrict__ big_count) {
    extern __shared__ uint32_t sseg[];  // BLOCK_CELL_MAX entries
    __shared__ uint32_t s_warp[BIG_THREADS / 32];
    uint32_t nbig = *big_count;
    if (nbig > BIG_LIST_CAP) nbig = BIG_LIST_CAP;
    for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
        const uint32_t c = big_list[b];
        const uint32_t n = count[c], off = offset[c];
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) work[off + k] = off + k;
        if (n <= (uint32_t)BLOCK_CELL_MAX) {
            for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) sseg[k] = order[off + k];
            __syncthreads();
            for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
                uint32_t x = sseg[k], r = 0;
                for (uint32_t m = 0; m < n; m++) r += sseg[m] < x ? 1u : 0u;
                sorted[off + r] = x;
                newidx[x] = off + r;
            }
            __syncthreads();
        } else {
            // Ordered stream compaction over all particles: members of cell c in index order.
            uint32_t running = 0;
            const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
            for (uint32_t base = 0; base < cap; base += blockDim.x) {
                uint32_t i = base + threadIdx.x;
                bool m = i < cap && cell[i] == c;
                unsigned bal = __ballot_sync(0xffffffffu, m);
                if (lane == 0) s_warp[warp] = (uint32_t)__popc(bal);
                __syncthreads();
                uint32_t before = 0, tot = 0;
                for (uint32_t q = 0; q < BIG_THREADS / 32; q++) {
                    if (q < warp) before += s_warp[q];
                    tot += s_warp[q];
                }
                if (m) {
                    uint32_t r = running + before + (uint32_t)__popc(bal & ((1u << lane) - 1u));
                    sorted[off + r] = i;
                    newidx[i] = off + r;
                }
                running += tot;
                __syncthreads();
            }
        }
    }
}

void launch_cellsort(const DevParams& P, const Scratch& s, int num_sms, bool subcounts,
                     cudaStream_t st) {
    const uint32_t blocks = (P.cap + 255) / 256;
    if (subcounts) cudaMemsetAsync(s.subcnt, 0, sizeof(unsigned long long) * P.cells, st);
    k_cellsort<<<blocks, 256, 0, st>>>(s.cell, s.count, s.offset, s.okey, s.sorted,
                                        s.newidx, s.work, subcounts ? s.subcnt : nullptr,
                                        s.big_list, s.counters + 1, s.counters + 2, s.counters + 3);
    k_cellsort_big<<<num_sms, BIG_THREADS, BLOCK_CELL_MAX * sizeof(uint32_t), st>>>(
        P.cap, s.cell, s.count, s.offset, s.order, s.sorted, s.newidx, s.work, s.big_list,
        s.counters + 1);
}

// ---- gather ---------------------------------------------------------------------------------
#ifndef MG_GATHER_V8
#define MG_GATHER_V8 1
#endif
// 32 bytes through one 256-bit access (both addresses 32-byte aligned: bond records are 32 bytes
// and concentration rows 64 bytes, in buffers aligned to 256 bytes).  The source set is not
// written by the gather, so its loads take the read-only path.
__device__ __forceinline__ void ld32(const void* src, uint4& a, uint4& b) {
#if MG_GATHER_V8
    asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
        : "l"(src));
#else
    a = __ldg(reinterpret_cast<const uint4*>(src));
    b = __ldg(reinterpret_cast<const uint4*>(src) + 1);
#endif
}
__device__ __forceinline__ void st32(void* dst, const uint4& a, const uint4& b) {
#if MG_GATHER_V8
    asm volatile("st.global.v8.u32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
                 ::"l"(dst), "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w)
                 : "memory");
#else
    reinterpret_cast<uint4*>(dst)[0] = a;
    reinterpret_cast<uint4*>(dst)[1] = b;
#endif
}
// a 64-byte concentration row
__device__ __forceinline__ void copy_row64(const float* src, float* dst) {
    uint4 a, b, c, d;
    ld32(src, a, b);
    ld32(src + 8, c, d);
    st32(dst, a, b);
    st32(dst + 8, c, d);
}

__device__ __forceinline__ uint32_t remap(uint32_t j, uint32_t cap, const uint32_t* newidx) {
    return j < cap ? __ldg(newidx + j) : NO_PARTNER;
}

__global__ void __launch_bounds__(MG_PLAIN_MAX_THREADS) k_gather(DevParams P, Carried S,
                                                const float* __restrict__ sconc, Carried D,
                                                float* __restrict__ dconc,
                                                const uint32_t* __restrict__ sorted,
                                                const uint32_t* __restrict__ newidx,
                                                const uint32_t* __restrict__ cell,
                                                uint32_t* __restrict__ scell,
                                                float4* __restrict__ force,
                                                const uint32_t* __restrict__ nactive_p,
                                                int parts, Cold cs, Cold cd) {
    // parts: GATHER_CORE (positions, genes, origins, cells, the bond partners; the scratch of
    // parked slots), GATHER_CONC (concentrations), GATHER_MOTION (velocities, incoming-bond
    // table).  The bond records stay at their origins; only their partners change, to this
    // sort's indices, in place.
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t cap = P.cap;
    if (p >= cap) return;
    if ((parts & GATHER_CORE) && !(parts & GATHER_REORIGIN)) {
        // slot p read as an origin: the six partners loaded first, then remapped and stored
        // (a store may alias the next slot's load as far as the compiler knows, which would
        // otherwise keep each slot's two loads waiting for the previous slot's store)
        uint32_t j[NB];
#pragma unroll
        for (int a = 0; a < NB; a++) j[a] = D.partner[bond_ip(cap, a, p)];
#pragma unroll
        for (int a = 0; a < NB; a++) j[a] = remap(j[a], cap, newidx);
#pragma unroll
        for (int a = 0; a < NB; a++) D.partner[bond_ip(cap, a, p)] = j[a];
    }
    const uint32_t nact = *nactive_p;
    if (p < nact) {
        const uint32_t i = checked(P, sorted[p], cap);
        if (parts & GATHER_CORE) {
            D.pos[p] = __ldg(S.pos + i);

            if (P.full_epi) {
                // per-gene words move with the particle; the bits (dense-list membership at sort
                // time, FEPIGEN > 0) are taken from them
                uint32_t bits = __ldg(S.genes + i) & 0x80000000u;
#pragma unroll
                for (int g = 0; g < NG; g++) {
                    const uint32_t wv = __ldg(S.epi + (size_t)g * cap + i);
                    D.epi[(size_t)g * cap + p] = wv;
                    if (wv != 0u) bits |= 1u << g;
                }
                D.genes[p] = bits;
            } else {
                D.genes[p] = __ldg(S.genes + i);
            }
            const uint32_t o0 = __ldg(S.origin + i), o = o0 == UNDEF ? UNDEF : checked(P, o0, cap);
            if (parts & GATHER_REORIGIN) {
                // the particle's records move to slot p of the other space, and p becomes its
                // origin (a particle without records keeps none)
                if (o != UNDEF) {
                    cd.age[p] = __ldg(cs.age + o);
                    cd.color[p] = __ldg(cs.color + o);
                    cd.pid[p] = __ldg(cs.pid + o);
                    cd.mass_radius[p] = __ldg(cs.mass_radius + o);
                    cd.nerve[p] = __ldg(cs.nerve + o);
#pragma unroll
                    for (int a = 0; a < NB; a++) {
                        cd.change[(size_t)p * NB + a] = __ldg(cs.change + (size_t)o * NB + a);
                        cd.bond[bond_ia(cap, a, p)] = __ldg(cs.bond + bond_ia(cap, a, o));
                        cd.bond[bond_ib(cap, a, p)] = __ldg(cs.bond + bond_ib(cap, a, o));
                        cd.partner[bond_ip(cap, a, p)] = remap(__ldg(cs.partner + bond_ip(cap, a, o)), cap, newidx);
                    }
                }
                D.origin[p] = o != UNDEF ? p : UNDEF;
            } else {
                D.origin[p] = o;
            }
            if (S.iid) D.iid[p] = __ldg(S.iid + i);
            scell[p] = __ldg(cell + i);
        }
        if (parts & GATHER_SCRATCH) {  // countingSortFull's FPRESS / FDENSITY copy, FFORCE = 0
            D.press[p] = __ldg(S.press + i);
            D.invdens[p] = __ldg(S.invdens + i);
            force[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if (parts & GATHER_MOTION) {
            D.vel[p] = __ldg(S.vel + i);
            D.veval[p] = __ldg(S.veval + i);
            const uint4* pi = reinterpret_cast<const uint4*>(S.pidx + (size_t)i * 12);
            uint4* po = reinterpret_cast<uint4*>(D.pidx + (size_t)p * 12);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                uint4 v = __ldg(pi + k);
                v.x = remap(v.x, cap, newidx);
                v.z = remap(v.z, cap, newidx);
                po[k] = v;
            }
        }
        if (parts & GATHER_CONC) copy_row64(sconc + (size_t)i * NTF, dconc + (size_t)p * NTF);
    } else {
        // parked null particle (out-of-grid parking of advanceParticles, cuda:3474-3477)
        if (parts & GATHER_CORE) {
            D.pos[p] = make_float4(P.bmin[0], P.bmin[1], P.null_z, 0.0f);

            D.genes[p] = 0u;
            if (P.full_epi)
                for (int g = 0; g < NG; g++) D.epi[(size_t)g * cap + p] = 0u;
            D.origin[p] = UNDEF;
            if (D.iid) D.iid[p] = UNDEF;
            scell[p] = UNDEF;
            D.press[p] = 0.f;
            D.invdens[p] = 0.f;
            force[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if (parts & GATHER_MOTION) {
            D.vel[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            D.veval[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            uint4* po = reinterpret_cast<uint4*>(D.pidx + (size_t)p * 12);
#pragma unroll
            for (int k = 0; k < 3; k++) po[k] = make_uint4(NO_PARTNER, NO_PARTNER, NO_PARTNER, NO_PARTNER);
        }
        if (parts & GATHER_CONC) {
            float4* co = reinterpret_cast<float4*>(dconc + (size_t)p * NTF);
#pragma unroll
            for (int k = 0; k < 4; k++) co[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

void launch_gather(const DevParams& P, const Carried& src, const float* src_conc,
                   const Carried& dst, float* dst_conc, const Scratch& s, cudaStream_t st,
                   int parts, const Cold* cs, const Cold* cd) {
    const uint32_t nt = (uint32_t)P.gather_threads, blocks = (P.cap + nt - 1) / nt;
    if ((parts & GATHER_REORIGIN) && (!cs || !cd || !(parts & GATHER_CORE))) parts &= ~GATHER_REORIGIN;
    k_gather<<<blocks, nt, 0, st>>>(P, src, src_conc, dst, dst_conc, s.sorted, s.newidx, s.cell,
                                      s.scell, s.force, s.counters + 3, parts,
                                      cs ? *cs : Cold{}, cd ? *cd : Cold{});
}

}  // namespace mg
