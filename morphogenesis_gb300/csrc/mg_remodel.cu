// mg_remodel.cu - re-forming of broken bonds (row a11, Run2Remodelling).
//
// Reference: heal (fluid_system_cuda.cu:2047-2105) with contribFindBonds' bond-0 rule
// (theta = dsq, cuda:1938-1975) and makeBond (cuda:1573-1593); breaks happen in computeForce
// (rest length set to 0, cuda:3315-3316).  The reference jitters the search point with curand
// (cuda:2066-2071) and lets every broken bond race for its partner's incoming slot 0.  Here the
// rule is deterministic, in three passes over the sorted particles of the current step (before
// integration, as Run() calls it before AdvanceCL):
//   free     : per particle, the mask of incoming slots that hold no live bond;
//   propose  : a particle with a broken slot (active partner, rest length failing the
//              computeForce test) proposes, for its lowest broken slot, the nearest particle
//              within h that is not a boundary marker (particle id 0), not already one of its
//              partners and has a free incoming slot; ties go to the lower sorted index;
//   accept   : each proposed-to particle takes proposals in (distance, index) order into its
//              free incoming slots in slot order; a taken proposal writes the new bond (rest
//              length = distance, elastic limit 1.5 x rest length, modulus and damping kept,
//              integrators 0, word 5 = partner's particle id) and the incoming entry.
// Compiled with -fmad=false: distances are the reference expression, bit for bit.
#include "mg_internal.cuh"

namespace mg {

namespace {

// (double)restlen < 1e-9 of computeForce (cuda:3268) as a float compare: 0x30897060 is the
// smallest float not below 1e-9.
__device__ __forceinline__ bool rest_is_small(uint32_t rest_bits) {
    return __uint_as_float(rest_bits) < __int_as_float(0x30897060);
}

__device__ __forceinline__ uint4 bond_a(const uint4* bond, uint32_t cap, uint32_t p, int a) {
    return bond[((size_t)a * cap + p) * 2];
}

__device__ __forceinline__ int lowest_broken_slot(const uint4* bond, uint32_t cap, uint32_t p,
                                                  uint32_t nact) {
#pragma unroll
    for (int a = 0; a < NB; a++) {
        const uint4 A = bond_a(bond, cap, p, a);
        if (A.x < nact && rest_is_small(A.y)) return a;
    }
    return -1;
}

__global__ void __launch_bounds__(256) k_free_slots(uint32_t cap, const uint4* __restrict__ bond,
                                                    const uint32_t* __restrict__ pidx,
                                                    const uint32_t* __restrict__ nactive_p,
                                                    uint8_t* __restrict__ freemask) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *nactive_p;
    if (j >= n) return;
    uint32_t m = 0;
#pragma unroll
    for (int s = 0; s < NB; s++) {
        const uint32_t k = pidx[(size_t)j * 12 + 2 * s], bk = pidx[(size_t)j * 12 + 2 * s + 1];
        bool live = false;
        if (k < n && bk < (uint32_t)NB) {
            const uint4 A = bond_a(bond, cap, k, (int)bk);
            live = A.x == j && !rest_is_small(A.y);
        }
        if (!live) m |= 1u << s;
    }
    freemask[j] = (uint8_t)m;
}

__global__ void __launch_bounds__(256) k_propose(DevParams P, const float4* __restrict__ pos,
                                                 const uint4* __restrict__ bond,
                                                 const uint32_t* __restrict__ origin,
                                                 const uint32_t* __restrict__ pid_cold,
                                                 const uint32_t* __restrict__ scell,
                                                 const uint32_t* __restrict__ count,
                                                 const uint32_t* __restrict__ offset,
                                                 const uint8_t* __restrict__ freemask,
                                                 const uint32_t* __restrict__ nactive_p,
                                                 uint32_t* __restrict__ prop,
                                                 float* __restrict__ propd) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *nactive_p;
    if (i >= n) return;
    const uint32_t cap = P.cap;
    prop[i] = UNDEF;
    propd[i] = 0.f;
    if (lowest_broken_slot(bond, cap, i, n) < 0) return;
    uint32_t partners[NB];
#pragma unroll
    for (int a = 0; a < NB; a++) partners[a] = bond_a(bond, cap, i, a).x;
    const float4 ip = pos[i];
    const uint32_t base = scell[i] - (uint32_t)P.nadj;
    float best = 0.f;
    uint32_t bj = UNDEF;
    for (int c = 0; c < P.adjcnt; c++) {
        const uint32_t cell = base + (uint32_t)P.adj[c];
        const uint32_t cnt = count[cell];
        if (cnt == 0) continue;
        const uint32_t off = offset[cell];
        for (uint32_t j = off; j < off + cnt; j++) {
            const float4 jp = pos[j];
            const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
            const float dsq = dx * dx + dy * dy + dz * dz;
            if (!(dsq < P.r2diff && dsq > 0.f)) continue;
            if (freemask[j] == 0) continue;
            bool bonded = false;
#pragma unroll
            for (int a = 0; a < NB; a++) bonded |= partners[a] == j;
            if (bonded) continue;
            const uint32_t o = origin[j];
            if (o == UNDEF || pid_cold[o] == 0u) continue;  // boundary marker particles
            if (bj == UNDEF || dsq < best) {
                best = dsq;
                bj = j;
            }
        }
    }
    prop[i] = bj;
    propd[i] = best;
}

__global__ void __launch_bounds__(256) k_accept(DevParams P, uint4* __restrict__ bond,
                                                uint32_t* __restrict__ pidx,
                                                const uint32_t* __restrict__ origin,
                                                const uint32_t* __restrict__ pid_cold,
                                                uint32_t* __restrict__ change_cold,
                                                const uint32_t* __restrict__ scell,
                                                const uint32_t* __restrict__ count,
                                                const uint32_t* __restrict__ offset,
                                                const uint8_t* __restrict__ freemask,
                                                const uint32_t* __restrict__ prop,
                                                const float* __restrict__ propd,
                                                const uint32_t* __restrict__ nactive_p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *nactive_p;
    if (i >= n) return;
    const uint32_t j = prop[i];
    if (j >= n) return;
    const float d = propd[i];
    const uint32_t cap = P.cap;
    uint32_t rank = 0;
    const uint32_t base = scell[j] - (uint32_t)P.nadj;
    for (int c = 0; c < P.adjcnt; c++) {
        const uint32_t cell = base + (uint32_t)P.adj[c];
        const uint32_t cnt = count[cell];
        const uint32_t off = cnt ? offset[cell] : 0u;
        for (uint32_t q = off; q < off + cnt; q++)
            if (prop[q] == j) {
                const float dq = propd[q];
                if (dq < d || (dq == d && q < i)) rank++;
            }
    }
    const uint32_t m = freemask[j];
    int slot = -1;
    uint32_t r = rank;
#pragma unroll
    for (int s = 0; s < NB; s++)
        if (slot < 0 && ((m >> s) & 1u)) {
            if (r == 0) slot = s;
            else r--;
        }
    if (slot < 0) return;  // no free incoming slot left for this proposal: retry next step
    const int b = lowest_broken_slot(bond, cap, i, n);
    if (b < 0) return;
    const size_t r0 = ((size_t)b * cap + i) * 2;
    const uint4 A = bond[r0];
    const float rest = sqrtf(d);
    const uint32_t oj = origin[j];
    bond[r0] = make_uint4(j, __float_as_uint(rest), A.z, A.w);
    bond[r0 + 1] = make_uint4(__float_as_uint(1.5f * rest), oj != UNDEF ? pid_cold[oj] : UNDEF, 0u, 0u);
    const uint32_t oi = origin[i];
    if (oi != UNDEF) change_cold[(size_t)oi * NB + b] = 0u;
    pidx[(size_t)j * 12 + 2 * slot] = i;
    pidx[(size_t)j * 12 + 2 * slot + 1] = (uint32_t)b;
}

}  // namespace

void launch_remodel(const DevParams& P, const Carried& cur, const Cold& cold, const Scratch& s,
                    cudaStream_t st) {
    const uint32_t blocks = (P.cap + 255) / 256;
    k_free_slots<<<blocks, 256, 0, st>>>(P.cap, cur.bond, cur.pidx, s.counters + 3, s.freemask);
    k_propose<<<blocks, 256, 0, st>>>(P, cur.pos, cur.bond, cur.origin, cold.pid, s.scell, s.count,
                                      s.offset, s.freemask, s.counters + 3, s.prop, s.propd);
    k_accept<<<blocks, 256, 0, st>>>(P, cur.bond, cur.pidx, cur.origin, cold.pid, cold.change,
                                     s.scell, s.count, s.offset, s.freemask, s.prop, s.propd,
                                     s.counters + 3);
}

}  // namespace mg
