// mg_io.cu - conversion between the reference buffer layouts (include/mg_abi.h) and the
// device layout, the index views FGCELL/FGNDX/FBIN, and the per-gene dense lists
// (countingSortDenseLists + tally_denselist_lengths, fluid_system_cuda.cu:185-194, 329-404).
#include "mg_internal.cuh"

namespace mg {

constexpr uint32_t EPIGEN_ACTIVE = 2147483647u;

static inline uint32_t blocks_for(size_t n) { return (uint32_t)((n + 255) / 256); }

// FELASTIDX word order: [0]partner [1]elastlim [2]restlen [3]modulus [4]damping [5]pid
// [6]strain^2 integrator [7]strain integrator [8]change type (fluid.h:73, 155).  The records
// live at the particle's origin; a slot without one (a particle dropped from the grid) keeps
// nothing, like the cold fields, and reads back as no bond.
__global__ void k_import_bonds(uint32_t cap, const uint32_t* __restrict__ ref,
                               uint4* __restrict__ bond, uint32_t* __restrict__ partner,
                               const uint32_t* __restrict__ origin, uint32_t* __restrict__ change) {
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)cap * NB) return;
    uint32_t p = (uint32_t)(k / NB), a = (uint32_t)(k % NB);
    const uint32_t* w = ref + k * 9;
    const uint32_t o = origin[p];
    if (o == UNDEF) return;
    bond[bond_ia(cap, (int)a, o)] = make_uint4(0u, w[2], w[3], w[4]);
    bond[bond_ib(cap, (int)a, o)] = make_uint4(w[1], w[5], w[6], w[7]);
    partner[bond_ip(cap, (int)a, o)] = w[0];
    change[(size_t)o * NB + a] = w[8];
}

__global__ void k_export_bonds(uint32_t cap, const uint4* __restrict__ bond,
                               const uint32_t* __restrict__ partner,
                               const uint32_t* __restrict__ origin,
                               const uint32_t* __restrict__ change,
                               const uint32_t* __restrict__ brk, int apply_breaks,
                               const uint32_t* __restrict__ nactive_p, uint32_t* __restrict__ ref) {
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)cap * NB) return;
    uint32_t p = (uint32_t)(k / NB), a = (uint32_t)(k % NB);
    const uint32_t o = origin[p];
    uint4 A = make_uint4(NO_PARTNER, 0u, 0u, 0u), B = make_uint4(0u, NO_PARTNER, 0u, 0u);
    if (o != UNDEF) {  // else a parked slot: no bond
        A = bond[bond_ia(cap, (int)a, o)];
        B = bond[bond_ib(cap, (int)a, o)];
        A.x = partner[bond_ip(cap, (int)a, o)];
    }
    if (apply_breaks && p < *nactive_p && (brk[p] >> a) & 1u) A.y = 0u;
    uint32_t* w = ref + k * 9;
    w[0] = A.x; w[1] = B.x; w[2] = A.y; w[3] = A.z; w[4] = A.w;
    w[5] = B.y; w[6] = B.z; w[7] = B.w;
    w[8] = o != UNDEF ? change[(size_t)o * NB + a] : 0u;
}

void launch_import_bonds(const DevParams& P, const uint32_t* ref, const Carried& cur,
                         const Cold& cold, cudaStream_t st) {
    size_t n = (size_t)P.cap * NB;
    k_import_bonds<<<blocks_for(n), 256, 0, st>>>(P.cap, ref, cur.bond, cur.partner, cur.origin, cold.change);
}

void launch_export_bonds(const DevParams& P, const Carried& cur, const Cold& cold,
                         const Scratch& s, bool apply_breaks, uint32_t* ref, cudaStream_t st) {
    size_t n = (size_t)P.cap * NB;
    k_export_bonds<<<blocks_for(n), 256, 0, st>>>(P.cap, cur.bond, cur.partner, cur.origin, cold.change, s.brk,
                                                   apply_breaks ? 1 : 0, s.counters + 3, ref);
}

// FEPIGEN [gene][particle] <-> gene bitmask.  Values other than 0 and INT_MAX carry an
// epigenetic countdown that the bitmask cannot hold; they raise ERR_EPIGEN_VALUE.
__global__ void k_import_epigen(uint32_t cap, const uint32_t* __restrict__ ref,
                                uint32_t* __restrict__ genes, uint32_t* __restrict__ err) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cap) return;
    uint32_t bits = 0;
    bool bad = false;
    for (int g = 0; g < NG; g++) {
        uint32_t v = ref[(size_t)g * cap + p];
        if (v != 0u) bits |= 1u << g;
        if (v != 0u && v != EPIGEN_ACTIVE) bad = true;
    }
    genes[p] = bits;
    if (bad) atomicOr(err, ERR_EPIGEN_VALUE);
}

__global__ void k_export_epigen(uint32_t cap, const uint32_t* __restrict__ genes,
                                uint32_t* __restrict__ ref) {
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)cap * NG) return;
    uint32_t g = (uint32_t)(k / cap), p = (uint32_t)(k % cap);
    ref[k] = ((genes[p] >> g) & 1u) ? EPIGEN_ACTIVE : 0u;
}

__global__ void k_bits_to_words(uint32_t cap, const uint32_t* __restrict__ genes, uint32_t* __restrict__ epi) {
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)cap * NG) return;
    uint32_t g = (uint32_t)(k / cap), p = (uint32_t)(k % cap);
    epi[k] = ((genes[p] >> g) & 1u) ? EPIGEN_ACTIVE : 0u;
}

// Gene bits (dense-list membership, FEPIGEN > 0) from the words; bit 31 is kept.
__global__ void k_words_to_bits(uint32_t cap, const uint32_t* __restrict__ epi, uint32_t* __restrict__ genes) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cap) return;
    uint32_t bits = genes[p] & 0x80000000u;
    for (int g = 0; g < NG; g++)
        if (epi[(size_t)g * cap + p] != 0u) bits |= 1u << g;
    genes[p] = bits;
}

void launch_bits_to_words(uint32_t cap, const Carried& c, cudaStream_t st) {
    k_bits_to_words<<<blocks_for((size_t)cap * NG), 256, 0, st>>>(cap, c.genes, c.epi);
}

void launch_words_to_bits(uint32_t cap, const Carried& c, cudaStream_t st) {
    k_words_to_bits<<<blocks_for(cap), 256, 0, st>>>(cap, c.epi, c.genes);
}

void launch_import_epigen(const DevParams& P, const uint32_t* ref, const Carried& cur,
                          uint32_t* err, cudaStream_t st) {
    k_import_epigen<<<blocks_for(P.cap), 256, 0, st>>>(P.cap, ref, cur.genes, err);
}

void launch_export_epigen(const DevParams& P, const Carried& cur, const Scratch& s, uint32_t* ref,
                          cudaStream_t st) {
    (void)s;
    size_t n = (size_t)P.cap * NG;
    k_export_epigen<<<blocks_for(n), 256, 0, st>>>(P.cap, cur.genes, ref);
}

__global__ void k_import_cold(uint32_t cap, const uint32_t* __restrict__ ref,
                              const uint32_t* __restrict__ origin, uint32_t* __restrict__ field) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cap) return;
    uint32_t o = origin[p];
    if (o != UNDEF) field[o] = ref[p];
}

__global__ void k_export_cold(uint32_t cap, const uint32_t* __restrict__ origin,
                              const uint32_t* __restrict__ field, uint32_t null_value,
                              uint32_t* __restrict__ ref) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cap) return;
    uint32_t o = origin[p];
    ref[p] = o != UNDEF ? field[o] : null_value;
}

void launch_import_cold(const DevParams& P, const uint32_t* ref, const Carried& cur,
                        uint32_t* cold_field, cudaStream_t st) {
    k_import_cold<<<blocks_for(P.cap), 256, 0, st>>>(P.cap, ref, cur.origin, cold_field);
}

void launch_export_cold(const DevParams& P, const Carried& cur, const Scratch& s,
                        const uint32_t* cold_field, uint32_t null_value, uint32_t* ref,
                        cudaStream_t st) {
    (void)s;
    k_export_cold<<<blocks_for(P.cap), 256, 0, st>>>(P.cap, cur.origin, cold_field, null_value, ref);
}

// which: 0 FGCELL, 1 FGNDX, 2 FBIN.  mode 1: indices of the pre-sort particles after
// insert; mode 2: sorted particles.
__global__ void k_export_grid_index(uint32_t cap, int which, int mode,
                                    const uint32_t* __restrict__ cell,
                                    const uint32_t* __restrict__ newidx,
                                    const uint32_t* __restrict__ scell,
                                    const uint32_t* __restrict__ offset,
                                    const uint32_t* __restrict__ nactive_p,
                                    uint32_t* __restrict__ ref) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cap) return;
    const uint32_t nact = *nactive_p;
    uint32_t v = UNDEF;
    if (which == 2) {
        v = p < nact ? p : UNDEF;
    } else if (mode == 1) {
        uint32_t c = cell[p];
        if (which == 0) v = c;
        else if (c != UNDEF) v = newidx[p] - offset[c];
    } else if (p < nact) {
        uint32_t c = scell[p];
        v = which == 0 ? c : p - offset[c];
    }
    ref[p] = v;
}

void launch_export_grid_index(const DevParams& P, const Scratch& s, int which, int mode,
                              uint32_t* ref, cudaStream_t st) {
    k_export_grid_index<<<blocks_for(P.cap), 256, 0, st>>>(P.cap, which, mode, s.cell, s.newidx,
                                                            s.scell, s.offset, s.counters + 3, ref);
}

// FCONC between the device's particle-major rows [N][16] and the species-major layout a
// reference host keeps (getConc(tf) = FCONC + tf * mMaxPoints, fluid_system.h:574): a 32 x 16
// tile through shared memory so that both sides are read and written coalesced.
__global__ void k_conc_transpose(uint32_t cap, const float* __restrict__ src, float* __restrict__ dst,
                                 int to_species_major) {
    __shared__ float tile[32][NTF + 1];
    const uint32_t p0 = blockIdx.x * 32u;
    const uint32_t tx = threadIdx.x & 31u, ty = threadIdx.x >> 5;  // 32 x 16 threads
    if (to_species_major) {
        for (uint32_t k = threadIdx.x; k < 32u * NTF; k += blockDim.x) {  // rows in
            const uint32_t r = k / NTF, t = k % NTF;
            if (p0 + r < cap) tile[r][t] = src[(size_t)(p0 + r) * NTF + t];
        }
        __syncthreads();
        if (p0 + tx < cap) dst[(size_t)ty * cap + p0 + tx] = tile[tx][ty];  // species rows out
    } else {
        if (p0 + tx < cap) tile[tx][ty] = src[(size_t)ty * cap + p0 + tx];
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < 32u * NTF; k += blockDim.x) {
            const uint32_t r = k / NTF, t = k % NTF;
            if (p0 + r < cap) dst[(size_t)(p0 + r) * NTF + t] = tile[r][t];
        }
    }
}

void launch_conc_transpose(uint32_t cap, const float* src, float* dst, bool to_species_major,
                           cudaStream_t st) {
    k_conc_transpose<<<(cap + 31) / 32, 32 * NTF, 0, st>>>(cap, src, dst, to_species_major ? 1 : 0);
}

__global__ void k_fill_u32(uint32_t* p, uint32_t v, size_t n) {
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] = v;
}

void launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st) {
    if (n) k_fill_u32<<<blocks_for(n), 256, 0, st>>>(p, v, n);
}

__global__ void k_identity(uint32_t* p, uint32_t n) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] = k;
}

void launch_identity(uint32_t* p, uint32_t n, cudaStream_t st) {
    if (n) k_identity<<<blocks_for(n), 256, 0, st>>>(p, n);
}

// ---- dense per-gene lists -------------------------------------------------------------------
__global__ void k_gene_cell_counts(uint32_t cap, uint32_t cells, const uint32_t* __restrict__ genes,
                                   const uint32_t* __restrict__ scell,
                                   const uint32_t* __restrict__ nactive_p,
                                   uint32_t* __restrict__ gcount) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p || p >= cap) return;
    uint32_t bits = genes[p] & 0xFFFFu, c = scell[p];
    while (bits) {
        int g = __ffs(bits) - 1;
        bits &= bits - 1;
        atomicAdd(&gcount[(size_t)g * cells + c], 1u);
    }
}

// List g holds the sorted indices of particles with gene g, bin by bin in ascending order
// (countingSortDenseLists writes lists[gene][offsets[gene][bin] + counter] in that order).
__global__ void k_gene_lists(uint32_t cap, uint32_t cells, const uint32_t* __restrict__ genes,
                             const uint32_t* __restrict__ scell,
                             const uint32_t* __restrict__ offset,
                             const uint32_t* __restrict__ goffset,
                             const uint32_t* __restrict__ nactive_p,
                             uint32_t* __restrict__ lists) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p || p >= cap) return;
    uint32_t bits = genes[p] & 0xFFFFu;
    if (!bits) return;
    uint32_t c = scell[p], start = offset[c];
    uint32_t before[NG];
#pragma unroll
    for (int g = 0; g < NG; g++) before[g] = 0;
    for (uint32_t q = start; q < p; q++) {
        uint32_t b = genes[q];
#pragma unroll
        for (int g = 0; g < NG; g++) before[g] += (b >> g) & 1u;
    }
#pragma unroll
    for (int g = 0; g < NG; g++)
        if ((bits >> g) & 1u) lists[(size_t)g * cap + goffset[(size_t)g * cells + c] + before[g]] = p;
}

void launch_gene_cell_counts(const DevParams& P, const Carried& cur, const Scratch& s,
                             uint32_t* gcount, cudaStream_t st) {
    k_gene_cell_counts<<<blocks_for(P.cap), 256, 0, st>>>(P.cap, P.cells, cur.genes, s.scell,
                                                           s.counters + 3, gcount);
}

void launch_gene_lists(const DevParams& P, const Carried& cur, const Scratch& s,
                       const uint32_t* goffset, uint32_t* lists, cudaStream_t st) {
    k_gene_lists<<<blocks_for(P.cap), 256, 0, st>>>(P.cap, P.cells, cur.genes, s.scell, s.offset,
                                                     goffset, s.counters + 3, lists);
}

}  // namespace mg

namespace mg {

// Fresh carried set: no bonds, no incoming bonds, identity origin.
__global__ void k_init_set(uint32_t cap, uint4* __restrict__ bond, uint32_t* __restrict__ partner,
                           uint32_t* __restrict__ pidx, uint32_t* __restrict__ origin) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cap) return;
    for (int a = 0; a < NB; a++) {  // slot p is origin p
        bond[bond_ia(cap, a, p)] = make_uint4(0u, 0u, 0u, 0u);
        bond[bond_ib(cap, a, p)] = make_uint4(0u, NO_PARTNER, 0u, 0u);
        partner[bond_ip(cap, a, p)] = NO_PARTNER;
    }
    for (int k = 0; k < 12; k++) pidx[(size_t)p * 12 + k] = NO_PARTNER;
    origin[p] = p;
}

void launch_init_set(uint32_t cap, const Carried& c, cudaStream_t st) {
    k_init_set<<<blocks_for(cap), 256, 0, st>>>(cap, c.bond, c.partner, c.pidx, c.origin);
}

}  // namespace mg
