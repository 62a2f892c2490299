// mg_remodel.cu - bond remodelling (row a11, Run2Remodelling): computeBondChanges, the change
// lists and the re-forming of broken bonds (heal).
//
// computeBondChanges (fluid_system_cuda.cu:1065-1331), over the living particles (gene 2, the
// dense list it is launched on): bond types from the tissue genes (bone 9: bonds 0-3 apatite;
// tendon 6 / muscle 7 / elastic ligament 10: bond 0 collagen; the cartilage branch tests gene 6
// again and is never taken, cuda:1127-1132); per bond in slot order, a bond with rest length > 0
// averages its strain integrators over the inner-loop steps, zeroes them and scales rest length
// and modulus by the genome's shifted tanh (cuda:1156-1207); its change word is zeroed; the first
// bond with rest length 0 or no partner is flagged for heal (change word 1) and ends the loop
// (cuda:1214-1244).  The lengthen / shorten / strengthen / weaken flags are never set by the
// reference (their insertion is commented out, cuda:1245-1285), so change lists 1-8 stay empty.
// tanh is mg_tanh_cw below, written from its definition so the oracle evaluates the same float
// operations.
//
// Change lists (countingSortChanges, cuda:406-618): bin by bin, the bin's particles in sorted
// order, each particle's bonds in slot order, one entry (particle, bond) per set bit of the
// bond's change word; built on demand for downloads.
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
//              integrators 0, word 5 = partner's particle id; or, with heal_params 1,
//              makeBond's elastin defaults from the genome) and the incoming entry.
// After computeBondChanges the slot a particle heals is its lowest slot in change list 0 that
// still needs a bond (rest length 0 or no active partner); otherwise its lowest slot whose
// partner is active and whose rest length failed the rest-length test.
// Compiled with -fmad=false: distances are the reference expression, bit for bit.
#include "mg_internal.cuh"
#include "mg_search.cuh"

namespace mg {

namespace {

// (double)restlen < 1e-9 of computeForce (cuda:3268) as a float compare: 0x30897060 is the
// smallest float not below 1e-9.
__device__ __forceinline__ bool rest_is_small(uint32_t rest_bits) {
    return __uint_as_float(rest_bits) < __int_as_float(0x30897060);
}

// Rest length bits and partner of bond slot a of the particle with origin o (its records'
// slot).
__device__ __forceinline__ uint32_t bond_rest(const uint4* bond, uint32_t cap, uint32_t o, int a) {
    return reinterpret_cast<const uint32_t*>(bond + bond_ia(cap, a, o))[1];
}

__device__ __forceinline__ int heal_slot(const uint4* bond, const uint32_t* partner, uint32_t cap,
                                         uint32_t p, uint32_t nact, const uint32_t* origin,
                                         const uint32_t* change, bool from_changes) {
    const uint32_t o = origin[p];
    if (o == UNDEF) return -1;
#pragma unroll
    for (int a = 0; a < NB; a++) {
        const uint32_t rest = bond_rest(bond, cap, o, a), j = partner[bond_ip(cap, a, o)];
        if (from_changes) {
            const uint32_t w = change[(size_t)o * NB + a];
            if ((w & 1u) && (__uint_as_float(rest) == 0.f || j >= nact)) return a;
        } else if (j < nact && rest_is_small(rest)) {
            return a;
        }
    }
    return -1;
}

__device__ __forceinline__ float fbits(uint32_t u) { return __uint_as_float(u); }

// tanh from its definition: |x| < 0.5, odd Taylor polynomial through x^15 (Horner in x^2);
// 0.5 <= |x| < 9, 1 - 2 / (exp(2|x|) + 1) with exp by Cody-Waite reduction (ln 2 split in a
// 16-bit head and a tail) and a degree-8 Taylor polynomial scaled by 2^k; beyond, +-1.
// Within 2 ulp of tanh; separate float operations (-fmad=false), as the oracle evaluates them.
__device__ float mg_tanh_cw(float x) {
    if (x != x) return x + x;
    const float ax = x < 0.0f ? -x : x;
    if (ax < 0.5f) {
        const float z = x * x;
        float t = fbits(0xbabed1b2u);
        t = t * z + fbits(0x3b6b69e8u);
        t = t * z + fbits(0xbc11371bu);
        t = t * z + fbits(0x3cb327a4u);
        t = t * z + fbits(0xbd5d0dd1u);
        t = t * z + fbits(0x3e088889u);
        t = t * z + fbits(0xbeaaaaabu);
        return x + x * (z * t);
    }
    if (ax < 9.0f) {
        const float y = ax + ax;
        const float k = rintf(y * fbits(0x3fb8aa3bu));
        const float r = (y - k * fbits(0x3f317200u)) - k * fbits(0x35bfbe8eu);
        float e = fbits(0x37d00d01u);
        e = e * r + fbits(0x39500d01u);
        e = e * r + fbits(0x3ab60b61u);
        e = e * r + fbits(0x3c088889u);
        e = e * r + fbits(0x3d2aaaabu);
        e = e * r + fbits(0x3e2aaaabu);
        e = e * r + 0.5f;
        e = e * r + 1.0f;
        e = e * r + 1.0f;
        e = e * fbits((uint32_t)((int)k + 127) << 23);
        const float t = 1.0f - 2.0f / (e + 1.0f);
        return x < 0.0f ? -t : t;
    }
    return x < 0.0f ? -1.0f : 1.0f;
}

__global__ void __launch_bounds__(256) k_bond_changes(DevParams P, const DevGenome* __restrict__ G,
                                                      Carried C, uint32_t* __restrict__ change_cold,
                                                      float steps,
                                                      const uint32_t* __restrict__ nactive_p) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *nactive_p;
    if (p >= n) return;
    const uint32_t bits = C.genes[p];
    if (!((bits >> 2) & 1u)) return;  // the living list (gene 2 at the sort)
    const size_t cap = P.cap;
    bool bone, fibre;
    if (C.epi) {  // the current words, as computeBondChanges reads FEPIGEN
        bone = C.epi[9 * cap + p] > 0u;
        fibre = C.epi[6 * cap + p] > 0u || C.epi[7 * cap + p] > 0u || C.epi[10 * cap + p] > 0u;
    } else {
        bone = (bits >> 9) & 1u;
        fibre = ((bits >> 6) & 1u) || ((bits >> 7) & 1u) || ((bits >> 10) & 1u);
    }
    const uint32_t o = C.origin[p];  // the bond records' slot
    if (o == UNDEF) return;
    for (int b = 0; b < NB; b++) {
        const int type = bone && b < 4 ? 2 : (fibre && b == 0 ? 1 : 0);
        const size_t ra = bond_ia((uint32_t)cap, b, o), rb = bond_ib((uint32_t)cap, b, o);
        uint4 A = C.bond[ra];
        float rest = __uint_as_float(A.y);
        if (rest > 0.f) {
            uint4 B = C.bond[rb];
            const float si = __uint_as_float(B.w) / steps, sq = __uint_as_float(B.z) / steps;
            const float* T = G->tanh_p[type];
            rest = rest * (T[0] + T[1] * mg_tanh_cw(T[2] * si - T[3]));
            const float mod = __uint_as_float(A.z) * (T[4] + T[5] * mg_tanh_cw(T[6] * sq - T[7]));
            A.y = __float_as_uint(rest);
            A.z = __float_as_uint(mod);
            B.z = 0u;
            B.w = 0u;
            C.bond[ra] = A;
            C.bond[rb] = B;
        }
        const bool heal = rest == 0.f || C.partner[bond_ip((uint32_t)cap, b, o)] >= n;
        change_cold[(size_t)o * NB + b] = heal ? 1u : 0u;
        if (heal) break;
    }
}

// Per cell and change list, the number of change-word bits set on its particles' bonds.
__global__ void __launch_bounds__(256) k_change_cell_counts(uint32_t cap, uint32_t cells,
                                                            const uint32_t* __restrict__ origin,
                                                            const uint32_t* __restrict__ change,
                                                            const uint32_t* __restrict__ scell,
                                                            const uint32_t* __restrict__ nactive_p,
                                                            uint32_t* __restrict__ ccount) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p || p >= cap) return;
    const uint32_t o = origin[p];
    if (o == UNDEF) return;
    const uint32_t c = scell[p];
    for (int b = 0; b < NB; b++) {
        uint32_t w = change[(size_t)o * NB + b] & ((1u << MG_NUM_CHANGES) - 1u);
        while (w) {
            const int k = __ffs(w) - 1;
            w &= w - 1;
            atomicAdd(&ccount[(size_t)k * cells + c], 1u);
        }
    }
}

// Entries of particle p: after those of the earlier particles of its cell, in bond order.
__global__ void __launch_bounds__(256) k_change_lists(uint32_t cap, uint32_t cells,
                                                      const uint32_t* __restrict__ origin,
                                                      const uint32_t* __restrict__ change,
                                                      const uint32_t* __restrict__ scell,
                                                      const uint32_t* __restrict__ offset,
                                                      const uint32_t* __restrict__ coffset,
                                                      const uint32_t* __restrict__ nactive_p,
                                                      uint32_t* __restrict__ lists) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p || p >= cap) return;
    const uint32_t o = origin[p];
    if (o == UNDEF) return;
    const uint32_t mask = (1u << MG_NUM_CHANGES) - 1u;
    uint32_t any = 0;
    for (int b = 0; b < NB; b++) any |= change[(size_t)o * NB + b] & mask;
    if (!any) return;
    const uint32_t c = scell[p];
    uint32_t before[MG_NUM_CHANGES];
#pragma unroll
    for (int k = 0; k < MG_NUM_CHANGES; k++) before[k] = 0;
    for (uint32_t q = offset[c]; q < p; q++) {
        const uint32_t oq = origin[q];
        if (oq == UNDEF) continue;
        for (int b = 0; b < NB; b++) {
            const uint32_t w = change[(size_t)oq * NB + b];
#pragma unroll
            for (int k = 0; k < MG_NUM_CHANGES; k++) before[k] += (w >> k) & 1u;
        }
    }
    for (int b = 0; b < NB; b++) {
        const uint32_t w = change[(size_t)o * NB + b] & mask;
#pragma unroll
        for (int k = 0; k < MG_NUM_CHANGES; k++)
            if ((w >> k) & 1u) {
                const size_t at = coffset[(size_t)k * cells + c] + before[k]++;
                lists[(size_t)k * 2 * cap + at] = p;
                lists[(size_t)k * 2 * cap + cap + at] = (uint32_t)b;
            }
    }
}

__global__ void __launch_bounds__(256) k_free_slots(uint32_t cap, const uint4* __restrict__ bond,
                                                    const uint32_t* __restrict__ partner,
                                                    const uint32_t* __restrict__ pidx,
                                                    const uint32_t* __restrict__ origin,
                                                    const uint32_t* __restrict__ pid_cold,
                                                    const uint32_t* __restrict__ nactive_p,
                                                    uint8_t* __restrict__ freemask) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *nactive_p;
    if (j >= n) return;
    const uint32_t o = origin[j];
    if (o == UNDEF || pid_cold[o] == 0u) {  // boundary markers (particle id 0) take no bond
        freemask[j] = 0;
        return;
    }
    uint32_t m = 0;
#pragma unroll
    for (int s = 0; s < NB; s++) {
        const uint32_t k = pidx[(size_t)j * 12 + 2 * s], bk = pidx[(size_t)j * 12 + 2 * s + 1];
        bool live = false;
        if (k < n && bk < (uint32_t)NB) {
            const uint32_t ok = origin[k];
            live = ok != UNDEF && partner[bond_ip(cap, (int)bk, ok)] == j &&
                   !rest_is_small(bond_rest(bond, cap, ok, (int)bk));
        }
        if (!live) m |= 1u << s;
    }
    freemask[j] = (uint8_t)m;
}

// Proposals (the propose pass above), found by the warp-cooperative search of the density pass: a warp takes
// 32 entries of the processing order (compact in space); the lanes that propose are searched in
// groups (a cell and the next of its row), each group's window cells are walked in ascending
// index, their particles loaded coalesced and kept when inside the group's box grown by h, and
// each proposing lane tests the kept ones of its own window cells with the exact distance
// expression, keeping the nearest eligible one (ties to the lower sorted index, as the serial
// walk in ascending index keeps the first).  A proposal is counted at its target and the first
// PROP_K proposers are listed there for the ranking in k_accept.
constexpr int PROPOSE_WARPS = 8;
__global__ void __launch_bounds__(PROPOSE_WARPS * 32) k_propose_warp(
    DevParams P, const float4* __restrict__ pos, const uint4* __restrict__ bond,
    const uint32_t* __restrict__ partner, const uint32_t* __restrict__ origin,
    const uint32_t* __restrict__ pid_cold,
    const uint32_t* __restrict__ scell, const uint32_t* __restrict__ count,
    const uint32_t* __restrict__ offset, const uint8_t* __restrict__ freemask,
    const uint32_t* __restrict__ nactive_p, const uint32_t* __restrict__ change, bool from_changes,
    const uint32_t* __restrict__ work, bool prune, const uint32_t* __restrict__ hcount,
    const uint32_t* __restrict__ hlist, uint32_t* __restrict__ prop, float* __restrict__ propd,
    uint32_t* __restrict__ prop_cnt, uint32_t* __restrict__ prop_list) {
    __shared__ float4 s_sp[PROPOSE_WARPS][32];
    __shared__ uint32_t s_sq[PROPOSE_WARPS][32];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *nactive_p;
    const bool act = k < n;
    const uint32_t cap = P.cap;
    const uint32_t i = act ? work[k] : 0u;
    if (act) {
        prop[i] = UNDEF;
        propd[i] = 0.f;
    }
    const bool wants = act && heal_slot(bond, partner, cap, i, n, origin, change, from_changes) >= 0;
    if (!__any_sync(0xffffffffu, wants)) return;
    uint32_t partners[NB];
    const uint32_t oi = wants ? origin[i] : UNDEF;
#pragma unroll
    for (int a = 0; a < NB; a++) partners[a] = wants ? partner[bond_ip(cap, a, oi)] : UNDEF;
    const float INF = __int_as_float(0x7f800000);
    const float4 ip = wants ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float best = 0.f;
    uint32_t bj = UNDEF;
    // a particle whose neighbours within h the density pass recorded takes them from there
    const uint32_t nh = wants && hcount ? hcount[k] : UNDEF;
    const bool need = wants && nh == UNDEF;
    if (wants && nh != UNDEF) {
        for (uint32_t t = 0; t < nh; t++) {
            const uint32_t j = hlist[(size_t)t * cap + k];
            const float4 jp = pos[j];
            const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
            const float dsq = dx * dx + dy * dy + dz * dz;
            if (!(dsq < P.r2diff && dsq > 0.f)) continue;
            if (bj != UNDEF && (dsq > best || (dsq == best && j > bj))) continue;
            if (freemask[j] == 0) continue;  // no free incoming slot, or a boundary marker
            bool bonded = false;
#pragma unroll
            for (int a = 0; a < NB; a++) bonded |= partners[a] == j;
            if (bonded) continue;
            best = dsq;
            bj = j;
        }
    }
    const uint32_t pcell = need ? scell[i] : 0u;
    const CellWin win = window_of(P, pcell);
    const float Rf = sqrtf(P.r2diff) * 1.0001f + 1e-3f;
    const int g = P.gsrch;
    const int BIG = 1 << 30;
    unsigned remaining = __ballot_sync(0xffffffffu, need);
    while (remaining) {
        const int leader = __ffs(remaining) - 1;
        const uint32_t lcell = __shfl_sync(0xffffffffu, pcell, leader);
        // the next cell is in the leader's row unless the leader's cell ends the row
        const bool row_next = __shfl_sync(0xffffffffu, win.x, leader) + 2 < P.res[0];
        const bool ing = need && ((remaining >> lane) & 1u) && pcell >= lcell && pcell - lcell <= 1u &&
                         (pcell == lcell || row_next);
        remaining &= ~__ballot_sync(0xffffffffu, ing);
        const float bx0 = warp_min(ing ? ip.x : INF) - Rf, bx1 = warp_max(ing ? ip.x : -INF) + Rf;
        const float by0 = warp_min(ing ? ip.y : INF) - Rf, by1 = warp_max(ing ? ip.y : -INF) + Rf;
        const float bz0 = warp_min(ing ? ip.z : INF) - Rf, bz1 = warp_max(ing ? ip.z : -INF) + Rf;
        const int wx0 = warp_mini(ing ? win.x : BIG), wx1 = warp_maxi(ing ? win.x : -BIG) + g - 1;
        const int wy0 = warp_mini(ing ? win.y : BIG), wy1 = warp_maxi(ing ? win.y : -BIG) + g - 1;
        const int wz0 = warp_mini(ing ? win.z : BIG), wz1 = warp_maxi(ing ? win.z : -BIG) + g - 1;
        const int ncx = wx1 - wx0 + 1, ncz = wz1 - wz0 + 1;
        const int ncell = ncx * ncz * (wy1 - wy0 + 1);
        for (int cb = 0; cb < ncell; cb += 32) {
            const int t = cb + (int)lane;
            uint32_t tcnt = 0, toff = 0, tpos = 0;  // tpos: the cell's offsets in the window
            if (t < ncell) {
                const int ox = t % ncx, oz = (t / ncx) % ncz, oy = t / (ncx * ncz);
                tpos = (uint32_t)ox | ((uint32_t)oy << 8) | ((uint32_t)oz << 16);
                const int cx = wx0 + ox, cz = wz0 + oz, cy = wy0 + oy;
                if (cx >= 0 && cy >= 0 && cz >= 0 && cx < P.res[0] && cy < P.res[1] && cz < P.res[2] &&
                    (!prune || cell_meets_box(P, cx, cy, cz, bx0, bx1, by0, by1, bz0, bz1))) {
                    const uint32_t cell = (uint32_t)((cy * P.res[2] + cz) * P.res[0] + cx);
                    tcnt = count[cell];
                    if (tcnt) toff = offset[cell];
                }
            }
            unsigned ne = __ballot_sync(0xffffffffu, tcnt != 0);
            while (ne) {
                const int src = __ffs(ne) - 1;
                ne &= ne - 1;
                const uint32_t cnt = __shfl_sync(0xffffffffu, tcnt, src);
                const uint32_t off = __shfl_sync(0xffffffffu, toff, src);
                const uint32_t pos3 = __shfl_sync(0xffffffffu, tpos, src);
                const int cx = wx0 + (int)(pos3 & 0xFFu), cy = wy0 + (int)((pos3 >> 8) & 0xFFu),
                          cz = wz0 + (int)(pos3 >> 16);
                const bool inw = ing && cx - win.x >= 0 && cx - win.x < g && cy - win.y >= 0 &&
                                 cy - win.y < g && cz - win.z >= 0 && cz - win.z < g;
                if (!__any_sync(0xffffffffu, inw)) continue;
                for (uint32_t base = 0; base < cnt; base += 32) {
                    const uint32_t kk = base + lane;
                    const bool valid = kk < cnt;
                    const float4 qp = valid ? pos[off + kk] : make_float4(INF, INF, INF, 0.f);
                    const bool surv = valid && qp.x >= bx0 && qp.x <= bx1 && qp.y >= by0 &&
                                      qp.y <= by1 && qp.z >= bz0 && qp.z <= bz1;
                    const unsigned ball = __ballot_sync(0xffffffffu, surv);
                    if (surv) {
                        const uint32_t slot = (uint32_t)__popc(ball & ((1u << lane) - 1u));
                        s_sp[w][slot] = qp;
                        s_sq[w][slot] = off + kk;
                    }
                    __syncwarp();
                    const int ns = __popc(ball);
                    if (inw) {
                        for (int tt = 0; tt < ns; tt++) {
                            const float4 jp = s_sp[w][tt];
                            const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
                            const float dsq = dx * dx + dy * dy + dz * dz;
                            if (!(dsq < P.r2diff && dsq > 0.f)) continue;
                            const uint32_t j = s_sq[w][tt];
                            if (bj != UNDEF && (dsq > best || (dsq == best && j > bj))) continue;
                            if (freemask[j] == 0) continue;  // no free slot, or a boundary marker
                            bool bonded = false;
#pragma unroll
                            for (int a = 0; a < NB; a++) bonded |= partners[a] == j;
                            if (bonded) continue;
                            best = dsq;
                            bj = j;
                        }
                    }
                    __syncwarp();
                }
            }
        }
    }
    if (wants) {
        prop[i] = bj;
        propd[i] = best;
        if (bj != UNDEF) {
            const uint32_t slot = atomicAdd(&prop_cnt[bj], 1u);
            if (slot < (uint32_t)PROP_K) prop_list[(size_t)bj * PROP_K + slot] = i;
        }
    }
}

__global__ void __launch_bounds__(256) k_accept(DevParams P, const DevGenome* __restrict__ G,
                                                uint4* __restrict__ bond,
                                                uint32_t* __restrict__ partner,
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
                                                const uint32_t* __restrict__ nactive_p,
                                                bool from_changes,
                                                const uint32_t* __restrict__ prop_cnt,
                                                const uint32_t* __restrict__ prop_list) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *nactive_p;
    if (i >= n) return;
    const uint32_t j = prop[i];
    if (j >= n) return;
    const float d = propd[i];
    const uint32_t cap = P.cap;
    uint32_t rank = 0;
    const uint32_t np = prop_cnt[j];
    if (np <= (uint32_t)PROP_K) {  // every proposer of j is listed
        for (uint32_t t = 0; t < np; t++) {
            const uint32_t q = prop_list[(size_t)j * PROP_K + t];
            const float dq = propd[q];
            if (dq < d || (dq == d && q < i)) rank++;
        }
    } else {  // more proposers than listed: the ones within h of j, found in its window
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
    const int b = heal_slot(bond, partner, cap, i, n, origin, change_cold, from_changes);
    if (b < 0) return;
    const uint32_t oi = origin[i];  // i's bond records' slot (valid: heal_slot found one)
    const size_t ra = bond_ia(cap, b, oi), rb = bond_ib(cap, b, oi);
    const uint4 A = bond[ra];
    const uint32_t oj = origin[j];
    const uint32_t pj = oj != UNDEF ? pid_cold[oj] : UNDEF;
    if (P.heal_params) {  // makeBond(i, j, b, slot, elastin) (cuda:1573-1593)
        const float* E = G->bparam[0];
        bond[ra] = make_uint4(0u, __float_as_uint(E[9]), __float_as_uint(E[10]), __float_as_uint(E[11]));
        bond[rb] = make_uint4(__float_as_uint(E[8]), pj, 0u, 0u);
    } else {
        const float rest = sqrtf(d);
        bond[ra] = make_uint4(0u, __float_as_uint(rest), A.z, A.w);
        bond[rb] = make_uint4(__float_as_uint(1.5f * rest), pj, 0u, 0u);
    }
    partner[bond_ip(cap, b, oi)] = j;
    change_cold[(size_t)oi * NB + b] = 0u;
    pidx[(size_t)j * 12 + 2 * slot] = i;
    pidx[(size_t)j * 12 + 2 * slot + 1] = (uint32_t)b;
}

}  // namespace

void launch_remodel(const DevParams& P, const DevGenome* G, const Carried& cur, const Cold& cold,
                    const Scratch& s, bool from_changes, bool prune, const uint32_t* hcount,
                    const uint32_t* hlist, cudaStream_t st) {
    const uint32_t blocks = (P.cap + 255) / 256;
    k_free_slots<<<blocks, 256, 0, st>>>(P.cap, cur.bond, cur.partner, cur.pidx, cur.origin, cold.pid, s.counters + 3,
                                         s.freemask);
    cudaMemsetAsync(s.prop_cnt, 0, sizeof(uint32_t) * P.cap, st);
    const uint32_t wblocks = (P.cap + PROPOSE_WARPS * 32 - 1) / (PROPOSE_WARPS * 32);
    k_propose_warp<<<wblocks, PROPOSE_WARPS * 32, 0, st>>>(
        P, cur.pos, cur.bond, cur.partner, cur.origin, cold.pid, s.scell, s.count, s.offset, s.freemask,
        s.counters + 3, cold.change, from_changes, s.work, prune, hcount, hlist, s.prop, s.propd,
        s.prop_cnt, s.prop_list);
    k_accept<<<blocks, 256, 0, st>>>(P, G, cur.bond, cur.partner, cur.pidx, cur.origin, cold.pid, cold.change,
                                     s.scell, s.count, s.offset, s.freemask, s.prop, s.propd,
                                     s.counters + 3, from_changes, s.prop_cnt, s.prop_list);
}

void launch_bond_changes(const DevParams& P, const DevGenome* G, const Carried& cur,
                         const Cold& cold, const Scratch& s, float steps, cudaStream_t st) {
    k_bond_changes<<<(P.cap + 255) / 256, 256, 0, st>>>(P, G, cur, cold.change, steps, s.counters + 3);
}

void launch_change_cell_counts(const DevParams& P, const Carried& cur, const Cold& cold,
                               const Scratch& s, uint32_t* ccount, cudaStream_t st) {
    k_change_cell_counts<<<(P.cap + 255) / 256, 256, 0, st>>>(P.cap, P.cells, cur.origin, cold.change,
                                                              s.scell, s.counters + 3, ccount);
}

void launch_change_lists(const DevParams& P, const Carried& cur, const Cold& cold,
                         const Scratch& s, const uint32_t* coffset, uint32_t* lists,
                         cudaStream_t st) {
    k_change_lists<<<(P.cap + 255) / 256, 256, 0, st>>>(P.cap, P.cells, cur.origin, cold.change,
                                                        s.scell, s.offset, coffset, s.counters + 3,
                                                        lists);
}

}  // namespace mg
