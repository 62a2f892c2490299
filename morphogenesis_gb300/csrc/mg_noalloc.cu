// mg_noalloc.cu - exclusive prefix sum over caller-owned device arrays that allocates nothing.
//
// Some callers are not allowed to allocate device memory when they need a scan: a host
// application that gives all of the GPU's memory to its own pool at start-up and allows no
// other allocation, code that runs inside an allocator's own callback (allocating there would
// re-enter the allocator), or a per-step loop that cannot accept the device-wide
// synchronisation that cudaFree performs.  mg_prefix_sum_cells needs a system made by
// mg_create, and mg_create allocates.  mg_prefix_sum_noalloc needs only the caller's own
// device arrays.
//
// The scan is the same single-pass decoupled look-back kernel that mg_prefix_sum_cells runs.
// Its scratch (one 64-bit status word per 4096-element tile, the tile ticket and an error
// word) lives in one fixed file-scope device array, so the input is limited to
// MG_NOALLOC_SCAN_MAX elements (16384 tiles, 128 KiB of scratch per device).  All calls on one
// device share that array: calls whose scans may overlap in time race on it.
#include <cstdio>

#include "../../include/mg_abi.h"
#include "mg_internal.cuh"

using namespace mg;

namespace {

constexpr uint32_t NOALLOC_TILES = 16384;
static_assert((uint64_t)NOALLOC_TILES * SCAN_TILE == MG_NOALLOC_SCAN_MAX,
              "scratch tiles and the declared maximum disagree");

// [0, NOALLOC_TILES): look-back status words.  [NOALLOC_TILES]: low 32 bits the tile ticket,
// high 32 bits the error word used when the caller passes none.
static __device__ __align__(256) unsigned long long g_scan_scratch[NOALLOC_TILES + 1];

// The scratch address in the current device's context.  It is looked up on every call (a host
// lookup, no device work): a cached address would outlive a cudaDeviceReset, after which the
// module and its scratch are loaded again at another address.
mg_status scratch_of_current_device(unsigned long long** out) {
    unsigned long long* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_scan_scratch);
    if (e != cudaSuccess || !p) {
        char msg[160];
        std::snprintf(msg, sizeof msg,
                      "mg_prefix_sum_noalloc: cudaGetSymbolAddress of the scratch: %s",
                      cudaGetErrorString(e));
        return record_thread_error(MG_ERR_CUDA, msg);
    }
    *out = p;
    return MG_OK;
}

}  // namespace

extern "C" mg_status mg_prefix_sum_noalloc(const uint32_t* counts, uint32_t* offsets, uint64_t n,
                                           uint32_t* total, uint32_t* error, void* stream) {
    if (n > MG_NOALLOC_SCAN_MAX) {
        char msg[200];
        std::snprintf(msg, sizeof msg,
                      "mg_prefix_sum_noalloc: n = %llu exceeds the maximum of %llu elements "
                      "that its fixed scratch holds", (unsigned long long)n,
                      (unsigned long long)MG_NOALLOC_SCAN_MAX);
        return record_thread_error(MG_ERR_INVALID_ARG, msg);
    }
    if (n > 0 && (!counts || !offsets))
        return record_thread_error(MG_ERR_INVALID_ARG,
                                   "mg_prefix_sum_noalloc: counts and offsets must be device "
                                   "pointers when n > 0");
    unsigned long long* scratch = nullptr;
    mg_status s = scratch_of_current_device(&scratch);
    if (s != MG_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t tiles = (uint32_t)scan_status_words((uint32_t)n);
    // Everything the look-back reads must start at zero: the status words of this call's
    // tiles, the ticket and the fallback error word.
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * tiles, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch + NOALLOC_TILES, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess && n == 0 && total) e = cudaMemsetAsync(total, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess && n > 0) {
        uint32_t* ticket = (uint32_t*)(scratch + NOALLOC_TILES);
        launch_scan(counts, offsets, (uint32_t)n, scratch, ticket, total,
                    error ? error : ticket + 1, st, /*narrow=*/true);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "mg_prefix_sum_noalloc: %s", cudaGetErrorString(e));
        return record_thread_error(MG_ERR_CUDA, msg);
    }
    return MG_OK;
}
