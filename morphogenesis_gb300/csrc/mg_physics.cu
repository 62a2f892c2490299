// mg_physics.cu - SPH density/pressure, diffusion + gene reaction, bond + fluid force and
// leap-frog integration (rows a6-a10).  Compiled with -fmad=false: every kernel evaluates the
// float operations of the reference kernels in their order, without fused multiply-adds, so
// results are reproducible bit for bit against the CPU restatement.
//
// Reference: contributePressure/computePressure (fluid_system_cuda.cu:620-712),
// contributeDiffusion/computeDiffusion (cuda:3026-3105), computeGeneAction/tallyGeneAction
// (cuda:714-772), contributeForce/computeForce (cuda:3167-3358), advanceParticles
// (cuda:3470-3614).
//
// Summation order.  The reference visits the gridAdj cells in ascending linear cell index and
// each cell's particles in sorted order, i.e. every neighbour sum runs over ascending sorted
// index q, with per-cell partial sums for density and fluid force.  Both search paths below
// keep exactly that order, so they give identical bits:
//  * direct: one thread per particle walks its gridAdjCnt cells (the reference loop);
//  * warp search: the 32 particles of a warp walk the union of their cell windows together.
//    Each chunk of 32 candidates is loaded once (one candidate per lane) and kept when it lies
//    within the search radius of the box spanned by the group's particles; survivors are
//    broadcast in ascending order and every lane appends the ones inside its own radius and
//    window to a per-lane list in shared memory.  The neighbour terms are then evaluated lane
//    by lane over these lists, so no lane idles through a neighbour that belongs to another
//    lane.  A lane whose list overflows (more than NL_CAP neighbours) is then walked by its
//    whole warp (the overflow walk, one warp per particle); the fine-cell search queues such
//    particles for the same walk in a second kernel.
// The density pass also records each particle's fluid-force neighbours (dsq < 1) so the force
// pass reads a short list instead of searching again.
#include <cfloat>
#include <cuda_bf16.h>
#include "mg_internal.cuh"
#include "mg_search.cuh"

namespace mg {

#ifndef MG_DENS_WARPS
#define MG_DENS_WARPS 8
#endif
#ifndef MG_DENS_MIN_BLOCKS
#define MG_DENS_MIN_BLOCKS 3
#endif
constexpr int DENS_WARPS = MG_DENS_WARPS;  // warps per block of the warp-cooperative pass
// rows of a lane's neighbour list in shared memory: the list appends are branch-free (every
// survivor is written at the next free row, only hits advance it); a batch of four survivors
// starts at row min(n, NL_CAP), so three spare rows take the writes past a full list
constexpr int NL_ROWS = NL_CAP + 4;

// ---- per-neighbour terms ---------------------------------------------------------------
// sr_inv_exact: 1 / sr when sr is a power of two, where the quotient r / sr is the product
// r * (1 / sr) exactly (a scaling by a power of two, rounded once either way); else 0
__device__ __forceinline__ float wendland_term(float dsq, float sr, float sr_inv_exact) {
    const float r = sqrtf(dsq);
    const float qq = sr_inv_exact != 0.f ? r * sr_inv_exact : r / sr;
    float b = 1.f - qq;
    b *= b;
    b *= b;
    return b * (4.f * qq + 1.f);
}

// Fluid-force list entries ([FL_CAP][cap], sorted particle indices < 2^31): the top bit marks
// the first entry of each grid cell, where the force pass flushes its per-cell partial sum.
constexpr uint32_t FLIST_CELL_START = 0x80000000u;

// Build switches kept for measuring each choice against its plain form (both forms give the
// same bits): 256-bit concentration rows, packed f32x2 diffusion terms (MG_F32X2 1: the species
// differences; 2: also the products and the sums, each as a fused operation rounding once).
#ifndef MG_ROW_V8
#define MG_ROW_V8 1
#endif
#ifndef MG_DENS_GENOME_BY_VALUE
#define MG_DENS_GENOME_BY_VALUE 1
#endif
#if MG_DENS_GENOME_BY_VALUE
#define MG_DENS_GENOME_PARAM const __grid_constant__ DevGenome Gv
#define MG_DENS_GENOME_ARG Gh
#else
#define MG_DENS_GENOME_PARAM const DevGenome* __restrict__ G
#define MG_DENS_GENOME_ARG G
#endif
#ifndef MG_F32X2
#define MG_F32X2 2
#endif
// A particle's 16 concentrations as two 256-bit loads: a gather of rows from 32 lanes then
// costs the L1 two accesses per row instead of four.  Rows are 64 bytes in buffers aligned to
// 256 bytes, so both halves are 32-byte aligned.
__device__ __forceinline__ void load_row16(const float* row, float (&v)[NTF]) {
    static_assert(NTF == 16, "rows of 16 concentrations");
#if MG_ROW_V8
    asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(row));
    asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8+32];"
        : "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
        : "l"(row));
#else
    const float4* r4 = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float4 x = r4[k];
        v[4 * k] = x.x; v[4 * k + 1] = x.y; v[4 * k + 2] = x.z; v[4 * k + 3] = x.w;
    }
#endif
}

// ... and stored as two 256-bit stores
__device__ __forceinline__ void store_row16(float* row, const float (&v)[NTF]) {
#if MG_ROW_V8
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
                 :: "l"(row), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                 : "memory");
    asm volatile("st.global.v8.f32 [%0+32], {%1, %2, %3, %4, %5, %6, %7, %8};"
                 :: "l"(row), "f"(v[8]), "f"(v[9]), "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
                 : "memory");
#else
    float4* r4 = reinterpret_cast<float4*>(row);
#pragma unroll
    for (int k = 0; k < 4; k++) r4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
#endif
}

// Neighbour q's concentrations into the diffusion sums (nc, when `diffuse`) and into the plain
// neighbour sum (ms, when MEAN).  (dif[t] * cc) * (cq[t] - cur[t]) is the reference term; with
// one common nonzero rate the product dif[t] * cc is the same value for every species.
template <bool DIFF, bool MEAN>
__device__ __forceinline__ void conc_terms_row(float (&nc)[NTF], float (&ms)[NTF], const float* __restrict__ dif,
                                               const float (&cur)[NTF], const float (&cj)[NTF],
                                               float cc, bool uniform, bool diffuse, float unit) {
    if (!DIFF && !MEAN) return;
#if MG_F32X2
    // Packed pairs of species (f32x2: two IEEE single operations, each rounded as the scalar
    // one) where no product feeds a sum: the compiler may fuse a packed multiply into the packed
    // add that consumes it, one rounding instead of the reference's two, so products and the
    // sums they feed stay scalar.
    if (MEAN) {
#pragma unroll
        for (int t = 0; t < NTF; t += 2) {
            const float2 r = __fadd2_rn(make_float2(ms[t], ms[t + 1]), make_float2(cj[t], cj[t + 1]));
            ms[t] = r.x; ms[t + 1] = r.y;
        }
    }
#else
    if (MEAN) {
#pragma unroll
        for (int t = 0; t < NTF; t++) ms[t] += cj[t];
    }
#endif
    if (DIFF && diffuse) {
        if (uniform) {
            const float a = dif[0] * cc;
#if MG_F32X2
            // cj - cur as cj + (-1) * cur: one rounding of the exact difference, as the
            // subtraction.  The packed __fmul2_rn and __fadd2_rn gave other bits than
            // __fmul_rn / __fadd_rn on random operands (45% of pairs, measured), with or without
            // a barrier between them, so the product and the sum are never written that way.
            const float2 m1 = make_float2(-1.f, -1.f);
#if MG_F32X2 >= 2
            // ... and the product and the sum as fused operations that round once each:
            // a * d + (-0) is the product a * d rounded (for every d, zeros' signs included),
            // p * unit + nc the sum p + nc rounded.  Three packed operations per species pair.
            // With a literal 1 for the unit the compiler fused the two into a * d + nc (one
            // rounding), even when written as inline fma.rn.f32x2; a unit read at run time it
            // cannot fold, and the probe of both forms on random operands (zeros, subnormals,
            // wide exponents) gave the scalar bits in every case.
            const float2 a2 = make_float2(a, a), one = make_float2(unit, unit), nz = make_float2(-0.f, -0.f);
#pragma unroll
            for (int t = 0; t < NTF; t += 2) {
                const float2 d = __ffma2_rn(make_float2(cur[t], cur[t + 1]), m1, make_float2(cj[t], cj[t + 1]));
                const float2 pr = __ffma2_rn(a2, d, nz);
                const float2 s = __ffma2_rn(pr, one, make_float2(nc[t], nc[t + 1]));
                nc[t] = s.x;
                nc[t + 1] = s.y;
            }
#else
#pragma unroll
            for (int t = 0; t < NTF; t += 2) {
                const float2 d = __ffma2_rn(make_float2(cur[t], cur[t + 1]), m1, make_float2(cj[t], cj[t + 1]));
                nc[t] += a * d.x;
                nc[t + 1] += a * d.y;
            }
#endif
#else
#pragma unroll
            for (int t = 0; t < NTF; t++) nc[t] += a * (cj[t] - cur[t]);
#endif
        } else {
#pragma unroll
            for (int t = 0; t < NTF; t++)
                if (dif[t] != 0.f) nc[t] += (dif[t] * cc) * (cj[t] - cur[t]);
        }
    }
}

// The same, loading neighbour q's row first.
template <bool DIFF, bool MEAN>
__device__ __forceinline__ void conc_terms(float (&nc)[NTF], float (&ms)[NTF], const float* __restrict__ dif,
                                           const float (&cur)[NTF], const float* conc, uint32_t q,
                                           float cc, bool uniform, bool diffuse, float unit) {
    if (!DIFF && !MEAN) return;
    float cj[NTF];
    load_row16(conc + (size_t)q * NTF, cj);
    conc_terms_row<DIFF, MEAN>(nc, ms, dif, cur, cj, cc, uniform, diffuse, unit);
}


// FLAGS: 1 density/pressure, 2 diffusion (+ decay), 4 gene reaction, 8 surrogate features,
// 16 capture of (features, reaction increment) pairs, 32 judge (the gene reaction runs only
// for the particles sampled this step or handed to the plain method and its result goes to
// conc_plain, while conc_out receives the diffused concentrations of every particle, to which
// the surrogate adds its predicted reaction increment).
template <int FLAGS>
struct DF {
    static constexpr bool DENS = FLAGS & 1, DIFF = FLAGS & 2, GENE = FLAGS & 4, FEAT = FLAGS & 8,
                          CAPTURE = FLAGS & 16, JUDGE = FLAGS & 32, MEAN = FEAT || CAPTURE;
};

// Slots past the active particles (parked: dropped from the grid) keep their concentrations
// through the morphogen stage, which writes the other buffer: their rows are copied across
// (the reference's per-particle loops skip them and leave them as they are).
template <int FLAGS>
__device__ __forceinline__ void park_conc(const float* conc_in, float* conc_out, uint32_t k,
                                          uint32_t nact, uint32_t cap) {
    using F = DF<FLAGS>;
    if ((F::DIFF || F::GENE || F::MEAN) && k >= nact && k < cap) {
        float v[NTF];
        load_row16(conc_in + (size_t)k * NTF, v);
        store_row16(conc_out + (size_t)k * NTF, v);
    }
}

__device__ __forceinline__ bool judged_lane(const DensExtra& X, uint32_t p, uint32_t gene_word) {
    if ((gene_word >> 31) & 1u) return true;  // handed to the plain method for good
    if (!X.judge_period || !X.judge_stride) return false;
    const uint32_t step = *X.step;
    if (step % X.judge_period) return false;
    return p % X.judge_stride == (step / X.judge_period) % X.judge_stride;
}

// The reference neighbour walk for one particle: density sum, diffusion and neighbour sums.
template <int FLAGS>
__device__ __forceinline__ float dens_direct(const DevParams& P, float4 ip, uint32_t pcell,
                                             const float4* __restrict__ pos,
                                             const float* __restrict__ conc,
                                             const uint32_t* __restrict__ count,
                                             const uint32_t* __restrict__ offset,
                                             float (&nc)[NTF], float (&ms)[NTF], uint32_t& mcnt,
                                             const float* __restrict__ dif, const float (&cur)[NTF],
                                             bool diffuse, uint32_t* __restrict__ flist = nullptr,
                                             uint32_t* __restrict__ fcount = nullptr,
                                             uint32_t p = 0) {
    using F = DF<FLAGS>;
    float sum = 0.f;
    uint32_t nf = 0;
    const uint32_t base = pcell - (uint32_t)P.nadj;
    for (int c = 0; c < P.adjcnt; c++) {
        const uint32_t cellc = base + (uint32_t)P.adj[c];
        const uint32_t cnt = count[cellc];
        if (cnt == 0) continue;
        const uint32_t off = offset[cellc];
        float part = 0.f;
        uint32_t fmark = FLIST_CELL_START;  // on this cell's first fluid-force neighbour
        for (uint32_t q = off; q < off + cnt; q++) {
            const float4 jp = pos[q];
            const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
            const float dsq = dx * dx + dy * dy + dz * dz;
            if (flist && dsq < 1.f && dsq > 0.f) {
                if (nf < (uint32_t)FL_CAP) flist[(size_t)nf * P.cap + p] = q | fmark;
                fmark = 0u;
                nf++;
            }
            if (F::DENS && dsq < P.r2 && dsq > 0.f) part += wendland_term(dsq, P.sr, P.sr_inv_exact);
            if ((F::DIFF || F::MEAN) && dsq < P.r2diff && dsq > 0.f) {
                conc_terms<F::DIFF, F::MEAN>(nc, ms, dif, cur, conc, q, (P.r2diff - dsq) * P.d2,
                                             false, diffuse, P.unit);
                mcnt++;
            }
        }
        if (F::DENS) sum += part;
    }
    if (fcount) fcount[p] = nf;
    return sum;
}

// The gene action with the full epigenetic state (computeGeneAction + tallyGeneAction,
// fluid_system_cuda.cu:714-772, with D3): for each gene in the particle's sort-time dense lists,
// in gene order, a counting-down word (0 < w < INT_MAX) is decremented and, when it reaches 0,
// starts the next active gene's countdown at its genome delay; the activity (sensitivity .
// concentrations) adds secretion and, above each activation threshold, one activation of the
// other gene.  Living particles (gene 2) add the secretion and the activations.  Kept out of
// line so it does not weigh on the registers of the common path.
__device__ __noinline__ void gene_action_full(const DevParams& P, const DevGenome* __restrict__ G,
                                              uint32_t p, uint32_t bits, const float (&c)[NTF],
                                              float (&cf)[NTF], uint32_t* __restrict__ epi) {
    const size_t cap = P.cap;
    uint32_t E[NG], dE[NG];
    float dc[NTF];
    for (int g = 0; g < NG; g++) { E[g] = epi[(size_t)g * cap + p]; dE[g] = 0u; }
    for (int t = 0; t < NTF; t++) dc[t] = 0.f;
    for (int g = 0; g < NG; g++) {
        if (!((bits >> g) & 1u)) continue;
        const int delay = (int)E[g];
        if (0 < delay && delay < 0x7FFFFFFF) {
            E[g]--;
            if (delay == 1 && g + 1 < NG && E[g + 1] != 0u) E[g + 1] = G->delay[g + 1];
        }
        float act = 0.f;
        for (int t = 0; t < NTF; t++) {
            const float sv = G->sens[g][t];
            if (sv != 0.f) act += sv * c[t];
        }
        const int ns = G->nsec[g];
        for (int k = 0; k < ns; k++) dc[G->sec_tf[g][k]] += G->sec_rate[g][k] * act;
        const int na = G->nact[g];
        for (int k = 0; k < na; k++)
            if (G->act_thr[g][k] < act) dE[G->act_gene[g][k]] += 1u;
    }
    const bool living = (bits & 4u) != 0u;
    for (int t = 0; t < NTF; t++) cf[t] = living ? c[t] + dc[t] : c[t];
    for (int g = 0; g < NG; g++) epi[(size_t)g * cap + p] = living ? E[g] + dE[g] : E[g];
}

// Density -> pressure and 1/density; diffusion + gene reaction (the plain update); surrogate
// features and captured training pairs.
template <int FLAGS>
__device__ __forceinline__ void dens_epilogue(const DevParams& P, const DevGenome* __restrict__ G,
                                              uint32_t p, float sum, const float (&nc)[NTF],
                                              const float (&ms)[NTF], uint32_t mcnt,
                                              const float (&cur)[NTF], bool plain,
                                              const uint32_t* __restrict__ genes,
                                              float* __restrict__ conc_out,
                                              float* __restrict__ press,
                                              float* __restrict__ invdens, const DensExtra& X) {
    using F = DF<FLAGS>;
    if (F::DENS) {
        sum = sum * P.pmass * P.wc2;
        if (sum == 0.f) sum = 1.f;
        press[p] = (sum - P.rest) * (X.iid ? P.inst[X.iid[p]].istiff : P.istiff);
        invdens[p] = 1.f / sum;
    }
    const uint32_t gene_word = (F::GENE || F::MEAN || F::JUDGE) ? genes[p] : 0u;
    if (!(F::DIFF || F::GENE || F::MEAN)) return;
    // concentrations after diffusion and decay (the reaction's input)
    float c[NTF];
#pragma unroll
    for (int t = 0; t < NTF; t++) c[t] = F::DIFF ? G->breakdown[t] * (cur[t] + nc[t]) : cur[t];
    float inv_s = 0.f;
    if (F::MEAN) {
        // surrogate inputs: the diffused concentrations and the neighbours' mean concentration,
        // both divided by the particle's scale, and the gene bits
        float sc = 0.f;
#pragma unroll
        for (int t = 0; t < NTF; t++) sc = fmaxf(sc, fabsf(c[t]));
        inv_s = sc > 0.f ? 1.f / sc : 0.f;  // all-zero concentrations: zero inputs and increment
        float f[MLP_FEATURES];
        const float inv = mcnt ? 1.f / (float)mcnt : 0.f;
#pragma unroll
        for (int t = 0; t < NTF; t++) {
            f[t] = c[t] * inv_s;
            f[NTF + t] = (mcnt ? ms[t] * inv : cur[t]) * inv_s;
            f[2 * NTF + t] = (float)((gene_word >> t) & 1u);
        }
        if (F::FEAT) {
            __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(X.feat + (size_t)p * MLP_FEATURES);
#pragma unroll
            for (int t = 0; t < MLP_FEATURES / 2; t++) o[t] = __floats2bfloat162_rn(f[2 * t], f[2 * t + 1]);
            X.feat_scale[p] = sc;
        }
        if (F::CAPTURE) {
            float4* o = reinterpret_cast<float4*>(X.cap_x + (size_t)p * MLP_FEATURES);
#pragma unroll
            for (int k = 0; k < MLP_FEATURES / 4; k++) o[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
        }
    }
    if (F::JUDGE) {  // every particle: diffused concentrations, the surrogate adds the reaction
        store_row16(conc_out + (size_t)p * NTF, c);
    }
    if (!F::GENE && !F::JUDGE) {  // diffusion only
        store_row16(conc_out + (size_t)p * NTF, c);
    }
    if (F::GENE && plain && P.full_epi && X.epi) {
        float cf[NTF];
        gene_action_full(P, G, p, gene_word & 0xFFFFu, c, cf, X.epi);
        float* dst = F::JUDGE ? X.conc_plain : conc_out;
        store_row16(dst + (size_t)p * NTF, cf);
        if (F::CAPTURE) {
            float4* y4 = reinterpret_cast<float4*>(X.cap_y + (size_t)p * NTF);
#pragma unroll
            for (int k = 0; k < 4; k++)
                y4[k] = make_float4((cf[4 * k] - c[4 * k]) * inv_s, (cf[4 * k + 1] - c[4 * k + 1]) * inv_s,
                                    (cf[4 * k + 2] - c[4 * k + 2]) * inv_s,
                                    (cf[4 * k + 3] - c[4 * k + 3]) * inv_s);
        }
    } else if (F::GENE && plain) {
        // Gene bits are the sort-time dense-list membership (FEPIGEN > 0).  With every
        // FEPIGEN in {0, INT_MAX} and no activation lists the countdown never fires and
        // the reaction is: for each active gene g in order, activity = sum_tf sens*conc,
        // secretion accumulates rate*activity; living particles (gene 2) add it.
        const uint32_t bits = gene_word & 0xFFFFu;
        float dc[NTF];
#pragma unroll
        for (int t = 0; t < NTF; t++) dc[t] = 0.f;
        for (int g = 0; g < NG; g++) {
            if (!((bits >> g) & 1u)) continue;
            float act = 0.f;
#pragma unroll
            for (int t = 0; t < NTF; t++) {
                const float sv = G->sens[g][t];
                if (sv != 0.f) act += sv * c[t];
            }
            const int ns = G->nsec[g];
            for (int k = 0; k < ns; k++) {
                const int tf = G->sec_tf[g][k];
                const float v = G->sec_rate[g][k] * act;
#pragma unroll
                for (int t = 0; t < NTF; t++)
                    if (t == tf) dc[t] += v;
            }
        }
        float cf[NTF];
#pragma unroll
        for (int t = 0; t < NTF; t++) cf[t] = (bits & 4u) ? c[t] + dc[t] : c[t];
        float* dst = F::JUDGE ? X.conc_plain : conc_out;
        store_row16(dst + (size_t)p * NTF, cf);
        if (F::CAPTURE) {
            float4* y4 = reinterpret_cast<float4*>(X.cap_y + (size_t)p * NTF);
#pragma unroll
            for (int k = 0; k < 4; k++)
                y4[k] = make_float4((cf[4 * k] - c[4 * k]) * inv_s, (cf[4 * k + 1] - c[4 * k + 1]) * inv_s,
                                    (cf[4 * k + 2] - c[4 * k + 2]) * inv_s,
                                    (cf[4 * k + 3] - c[4 * k + 3]) * inv_s);
        }
    }
}

template <int FLAGS>
__device__ __forceinline__ void load_conc(const DevGenome* __restrict__ G, const float* conc_in,
                                          uint32_t p, float (&cur)[NTF]) {
    using F = DF<FLAGS>;
    if (F::DIFF || F::GENE || F::MEAN) {
        load_row16(conc_in + (size_t)p * NTF, cur);
    }
}

// ---- direct kernel (one thread per particle, the reference loop) ------------------------
template <int FLAGS>
__global__ void __launch_bounds__(256) k_dens(DevParams P, const DevGenome* __restrict__ G,
                                              const float4* __restrict__ pos,
                                              const float* __restrict__ conc_in,
                                              float* __restrict__ conc_out,
                                              const uint32_t* __restrict__ genes,
                                              const uint32_t* __restrict__ scell,
                                              const uint32_t* __restrict__ count,
                                              const uint32_t* __restrict__ offset,
                                              float* __restrict__ press,
                                              float* __restrict__ invdens,
                                              const uint32_t* __restrict__ nactive_p, DensExtra X) {
    using F = DF<FLAGS>;
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p) {
        park_conc<FLAGS>(conc_in, conc_out, p, *nactive_p, P.cap);
        return;
    }
    float cur[NTF], nc[NTF], ms[NTF];
    load_conc<FLAGS>(G, conc_in, p, cur);
    const float* dif = G->diff;  // the species' rates, read from the genome where used
#pragma unroll
    for (int t = 0; t < NTF; t++) { nc[t] = 0.f; ms[t] = 0.f; }
    const bool plain = !F::JUDGE || judged_lane(X, p, genes[p]);
    uint32_t mcnt = 0;
    float sum = 0.f;
    if (F::DENS || F::DIFF || F::MEAN)
        sum = dens_direct<FLAGS>(P, pos[p], scell[p], pos, conc_in, count, offset, nc, ms, mcnt, dif,
                                 cur, true);
    dens_epilogue<FLAGS>(P, G, p, sum, nc, ms, mcnt, cur, plain, genes, conc_out, press, invdens, X);
}

// ---- warp-cooperative kernel ----------------------------------------------------------------
// List entries are sorted particle indices (< 2^31); the top bit marks the first entry of a
// lane's list that lies in a new grid cell, where the per-cell partial sum is flushed.
constexpr uint32_t LIST_CELL_START = 0x80000000u;

// Evaluates a lane's neighbour list (ascending sorted index, first entry of each cell flagged)
// with the reference expressions: density partial sums per cell, diffusion and neighbour sums,
// the fluid-force list; then the common epilogue.
template <int FLAGS>
__device__ __forceinline__ void dens_list_finish(
    const DevParams& P, const DevGenome* __restrict__ G, uint32_t p, float4 ip, uint32_t n,
    const uint32_t* my, const float4* __restrict__ pos, const float* __restrict__ conc_in,
    float* __restrict__ conc_out, const uint32_t* __restrict__ genes, float* __restrict__ press,
    float* __restrict__ invdens, uint32_t* __restrict__ flist, uint32_t* __restrict__ fcount,
    const DensExtra& X, uint32_t slot) {
    // slot: the particle's position in the processing order (where its re-forming candidates go)
    using F = DF<FLAGS>;
    float cur[NTF], nc[NTF], ms[NTF];
    load_conc<FLAGS>(G, conc_in, p, cur);
    const float* dif = G->diff;  // the species' rates, read from the genome where used
#pragma unroll
    for (int t = 0; t < NTF; t++) { nc[t] = 0.f; ms[t] = 0.f; }
    const bool plain = !F::JUDGE || judged_lane(X, p, genes[p]);
    uint32_t mcnt = 0;
    float sum = 0.f;
    {
        float part = 0.f;
        uint32_t nf = 0, nh = 0, fmark = 0u;
        for (uint32_t k = 0; k < n; k++) {
            const uint32_t e = my[k * 32];
            const uint32_t q = checked(P, e & ~LIST_CELL_START, P.cap);
            // the neighbour's row is loaded with its position (both depend on q alone), so the
            // two loads overlap; entries beyond the diffusion radius leave it unused.  Not in
            // the surrogate's forms, whose 16 neighbour sums leave no registers for it (spills)
            constexpr bool EARLY = F::DIFF && !F::MEAN;
            float cj[NTF];
            if (EARLY) load_row16(conc_in + (size_t)q * NTF, cj);
            const float4 jp = pos[q];
            if (e & LIST_CELL_START) {  // first neighbour of the next cell:
                if (F::DENS) {          // flush the previous cell's partial sum
                    sum += part;
                    part = 0.f;
                }
                fmark = FLIST_CELL_START;
            }
            const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
            const float dsq = dx * dx + dy * dy + dz * dz;
            if (dsq < 1.f && dsq > 0.f) {  // fluid-force neighbour, kept for the force pass
                if (nf < (uint32_t)FL_CAP) flist[(size_t)nf * P.cap + p] = q | fmark;
                fmark = 0u;
                nf++;
            }
            if (F::DENS && dsq < P.r2 && dsq > 0.f) part += wendland_term(dsq, P.sr, P.sr_inv_exact);
            if ((F::DIFF || F::MEAN) && dsq < P.r2diff && dsq > 0.f) {
                if (!EARLY) load_row16(conc_in + (size_t)q * NTF, cj);
                conc_terms_row<F::DIFF, F::MEAN>(nc, ms, dif, cur, cj, (P.r2diff - dsq) * P.d2,
                                                 G->uniform != 0, true, P.unit);
                mcnt++;
                if (X.hlist) X.hlist[(size_t)nh++ * P.cap + slot] = q;  // nh <= n <= NL_CAP
            }
        }
        if (F::DENS) sum += part;
        fcount[p] = nf;  // > FL_CAP: the force pass searches again
        if (X.hlist) X.hcount[slot] = nh;
    }
    dens_epilogue<FLAGS>(P, G, p, sum, nc, ms, mcnt, cur, plain, genes, conc_out, press, invdens, X);
}

// ---- overflow walk ----------------------------------------------------------------------------
// Particles with more neighbours than NL_CAP (only in dense clumps), one warp per particle
// (the warp search's own warp, or k_dens_ovf for the fine-cell search's queue), in two phases
// that repeat over segments of OVF_SEG hits:
//  collect : the window cells (in the reference order, 32 at a time, one per lane) form one
//            stream of candidates; each lane takes one candidate per chunk (its cell found by a
//            binary search over the cells' running counts), several chunks in flight, and the
//            hits are compacted in order into shared memory with their distance, window-cell
//            index and concentrations;
//  apply   : the hits are taken in that order by every lane: the density partial sum of each
//            cell, species t (mod 16) of the diffusion and neighbour sums in lane t with the
//            one-thread walk's expression and order, the force list in lane 0.
// Lane 0 then runs the common epilogue.
constexpr int OVF_SEG = 64;

// Takes a segment's hits in order (the apply phase of the overflow walk).
template <int FLAGS>
__device__ __forceinline__ void ovf_apply(const DevParams& P, uint32_t p, uint32_t lane, uint32_t t,
                                          uint32_t* __restrict__ flist, const float* sd,
                                          const uint32_t* sq, const uint8_t* sc, const float4 (*scj)[NTF / 4],
                                          uint32_t nh, int& lastcell, uint32_t& fmark, float& sum, float& part,
                                          uint32_t& nf, float& nc_t, float& ms_t, uint32_t& mcnt,
                                          float dif_t, float cur_t) {
    using F = DF<FLAGS>;
    __syncwarp();
    for (uint32_t h = 0; h < nh; h++) {
        const float d = sd[h];
        const int c = sc[h];
        if (c != lastcell) {  // first hit of the next cell: flush the previous partial
            sum += part;
            part = 0.f;
            lastcell = c;
            fmark = FLIST_CELL_START;
        }
        if (d < 1.f) {
            if (lane == 0 && nf < (uint32_t)FL_CAP) flist[(size_t)nf * P.cap + p] = sq[h] | fmark;
            fmark = 0u;
            nf++;
        }
        if (F::DENS && d < P.r2) part += wendland_term(d, P.sr, P.sr_inv_exact);
        if ((F::DIFF || F::MEAN) && d < P.r2diff) {
            const float cj = reinterpret_cast<const float*>(scj[h])[t];
            if (F::MEAN) ms_t += cj;
            if (F::DIFF && dif_t != 0.f) nc_t += (dif_t * ((P.r2diff - d) * P.d2)) * (cj - cur_t);
            mcnt++;
        }
    }
    __syncwarp();
}

// One queued particle, by the whole warp: s_cj, s_d, s_q and s_c hold a segment of OVF_SEG hits
// (OVF_SEG * 73 bytes of the warp's own shared memory).
template <int FLAGS, bool PACKED>
__device__ __forceinline__ void ovf_particle(
    const DevParams& P, const DevGenome* __restrict__ G0, uint32_t p, const float4* __restrict__ pos,
    const float* __restrict__ conc_in, float* __restrict__ conc_out, const uint32_t* __restrict__ genes,
    const uint32_t* __restrict__ scell, const uint32_t* __restrict__ count,
    const uint32_t* __restrict__ offset, float* __restrict__ press, float* __restrict__ invdens,
    uint32_t* __restrict__ flist, uint32_t* __restrict__ fcount, const DensExtra& X, bool prune,
    float4 (*s_cj)[NTF / 4], float* s_d, uint32_t* s_q, uint8_t* s_c) {
    // prune: positions are those of the last sort, so a window cell whose geometric box misses
    // the particle's search box holds no neighbour
    using F = DF<FLAGS>;
    constexpr bool CONC = F::DIFF || F::MEAN;
    const uint32_t lane = threadIdx.x & 31u, t = lane & 15u;
    float R2 = 1.f;
    if (F::DENS) R2 = fmaxf(R2, P.r2);
    if (CONC) R2 = fmaxf(R2, P.r2diff);
    const float Rf = sqrtf(R2) * 1.0001f + 1e-3f;  // conservative search-box half width
    const float4 ip = pos[p];
    const DevGenome* __restrict__ G = PACKED ? P.genomes + X.iid[p] : G0;
    const CellFrame frame = PACKED ? frame_of(P, X.iid[p]) : frame_of(P);
    const float cur_t = (F::DIFF || F::GENE || F::MEAN) ? conc_in[(size_t)p * NTF + t] : 0.f;
    const float dif_t = F::DIFF ? G->diff[t] : 0.f;
    const bool plain = !F::JUDGE || judged_lane(X, p, genes[p]);
    float nc_t = 0.f, ms_t = 0.f, sum = 0.f, part = 0.f;
    uint32_t mcnt = 0, nf = 0;
    int lastcell = -1;
    uint32_t fmark = 0u;
    const uint32_t base = scell[p] - (uint32_t)P.nadj;
    uint32_t nh = 0;  // hits of the current segment
    for (int cg = 0; cg < P.adjcnt; cg += 32) {
        // this group's window cells: count, offset and running start, one per lane
        const int ci = cg + (int)lane;
        uint32_t cnt = 0, off = 0;
        if (ci < P.adjcnt) {
            const uint32_t cellc = base + (uint32_t)P.adj[ci];
            const int cx = (int)(cellc % (uint32_t)P.res[0]);
            const int cz = (int)((cellc / (uint32_t)P.res[0]) % (uint32_t)P.res[2]);
            const int cy = (int)(cellc / ((uint32_t)P.res[0] * (uint32_t)P.res[2]));
            if (!prune || cell_meets_box(frame, cx, cy, cz, ip.x - Rf, ip.x + Rf, ip.y - Rf, ip.y + Rf,
                                         ip.z - Rf, ip.z + Rf)) {
                cnt = count[cellc];
                if (cnt) off = offset[cellc];
            }
        }
        uint32_t incl = cnt;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, dd);
            if ((int)lane >= dd) incl += v;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const uint32_t start = incl - cnt;
        for (uint32_t b0 = 0; b0 < total; b0 += 128) {
            // four chunks of 32 candidates in flight
            float dq[4];
            uint32_t qq[4], cc[4];
            bool hit[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t k = b0 + (uint32_t)u * 32u + lane;
                hit[u] = false;
                dq[u] = 0.f;
                qq[u] = 0u;
                cc[u] = 0u;
                // the cell holding candidate k: the last lane whose start is <= k
                uint32_t lo = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const uint32_t st = __shfl_sync(0xffffffffu, start, (int)(lo + step) & 31);
                    if (lo + step < 32 && st <= k) lo += step;
                }
                if (k < total) {
                    const uint32_t sl = __shfl_sync(0xffffffffu, start, (int)lo);
                    const uint32_t ol = __shfl_sync(0xffffffffu, off, (int)lo);
                    qq[u] = ol + (k - sl);
                    cc[u] = (uint32_t)cg + lo;
                } else {
                    __shfl_sync(0xffffffffu, start, (int)lo);
                    __shfl_sync(0xffffffffu, off, (int)lo);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t k = b0 + (uint32_t)u * 32u + lane;
                if (k < total) {
                    const float4 jp = pos[qq[u]];
                    const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
                    dq[u] = dx * dx + dy * dy + dz * dz;
                    hit[u] = dq[u] < R2 && dq[u] > 0.f;
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const unsigned ball = __ballot_sync(0xffffffffu, hit[u]);
                const uint32_t nb = (uint32_t)__popc(ball);
                if (nh + nb > (uint32_t)OVF_SEG) {  // segment full: take what it holds
                    ovf_apply<FLAGS>(P, p, lane, t, flist, s_d, s_q, s_c, s_cj, nh,
                                     lastcell, fmark, sum, part, nf, nc_t, ms_t, mcnt, dif_t, cur_t);
                    nh = 0;
                }
                if (hit[u]) {
                    const uint32_t slot = nh + (uint32_t)__popc(ball & ((1u << lane) - 1u));
                    s_d[slot] = dq[u];
                    s_q[slot] = qq[u];
                    s_c[slot] = (uint8_t)cc[u];
                    if (CONC && dq[u] < P.r2diff) {
                        const float4* c4 = reinterpret_cast<const float4*>(conc_in + (size_t)qq[u] * NTF);
#pragma unroll
                        for (int k4 = 0; k4 < NTF / 4; k4++) s_cj[slot][k4] = c4[k4];
                    }
                }
                nh += nb;
            }
        }
    }
    ovf_apply<FLAGS>(P, p, lane, t, flist, s_d, s_q, s_c, s_cj, nh, lastcell,
                     fmark, sum, part, nf, nc_t, ms_t, mcnt, dif_t, cur_t);
    if (F::DENS) sum += part;
    float cur[NTF], nc[NTF], ms[NTF];
#pragma unroll
    for (int k = 0; k < NTF; k++) {
        cur[k] = __shfl_sync(0xffffffffu, cur_t, k);
        nc[k] = __shfl_sync(0xffffffffu, nc_t, k);
        ms[k] = __shfl_sync(0xffffffffu, ms_t, k);
    }
    if (lane == 0) {
        fcount[p] = nf;
        dens_epilogue<FLAGS>(P, G, p, sum, nc, ms, mcnt, cur, plain, genes, conc_out, press,
                             invdens, X);
    }
    __syncwarp();
}

// Bytes of a warp's shared memory that ovf_particle takes.
constexpr size_t OVF_SMEM = (size_t)OVF_SEG * (NTF * sizeof(float) + sizeof(float) + sizeof(uint32_t) + 1);

// PACKED: packed instances (each particle's frame, genome and stiffness from its instance);
// a separate instantiation so that a single system keeps its genome in the constant bank.
template <int FLAGS, bool PACKED = false>
__global__ void __launch_bounds__(DENS_WARPS * 32, MG_DENS_MIN_BLOCKS) k_dens_warp(
    DevParams P, MG_DENS_GENOME_PARAM, const float4* __restrict__ pos,
    const float* __restrict__ conc_in, float* __restrict__ conc_out,
    const uint32_t* __restrict__ genes, const uint32_t* __restrict__ scell,
    const uint32_t* __restrict__ count, const uint32_t* __restrict__ offset,
    float* __restrict__ press, float* __restrict__ invdens, uint32_t* __restrict__ flist,
    uint32_t* __restrict__ fcount, const uint32_t* __restrict__ nactive_p,
    const uint32_t* __restrict__ work, DensExtra X, bool prune) {
    // prune: the positions are those of the last sort, so a window cell whose geometric box
    // misses the group's box holds no candidate; after positions moved, every cell is walked
    using F = DF<FLAGS>;
#if MG_DENS_GENOME_BY_VALUE
    const DevGenome* __restrict__ G = &Gv;  // the parameter itself: reads go to the constant bank
#endif
    extern __shared__ __align__(16) uint32_t s_list[];  // [warps of the block][NL_ROWS][32]
    static_assert(OVF_SMEM <= (size_t)NL_ROWS * 32 * sizeof(uint32_t), "overflow segment in a warp's list rows");
    // staged survivors, one array per coordinate so that four consecutive survivors' x (y, z,
    // sorted index) are one 128-bit load and pairs of them feed packed f32x2 operations
    __shared__ __align__(16) float s_sx[DENS_WARPS][32];
    __shared__ __align__(16) float s_sy[DENS_WARPS][32];
    __shared__ __align__(16) float s_sz[DENS_WARPS][32];
    __shared__ __align__(16) uint32_t s_sq[DENS_WARPS][32];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t* my = s_list + (size_t)w * NL_ROWS * 32 + lane;
    // Lane k of the grid takes the k-th entry of the processing order, so a warp holds
    // particles of one compact sub-region of a cell; results go to the particle's sorted slot.
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = k < *nactive_p;
    if (!act) park_conc<FLAGS>(conc_in, conc_out, k, *nactive_p, P.cap);
    if (!__any_sync(0xffffffffu, act)) return;
    const uint32_t p = act ? checked(P, work[k], P.cap) : 0u;

    const float4 ip = act ? pos[p] : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t pcell = act ? scell[p] : 0u;
    const CellWin win = window_of(P, pcell);
    // search radius: the largest threshold any term of this pass (and the force list) uses
    float R2 = 1.f;
    if (F::DENS) R2 = fmaxf(R2, P.r2);
    if (F::DIFF || F::MEAN) R2 = fmaxf(R2, P.r2diff);
    const float Rf = sqrtf(R2) * 1.0001f + 1e-3f;  // conservative prefilter radius
    const float R2s = R2 * 1.000004f;               // list threshold for the fused distance
    const float INF = __int_as_float(0x7f800000);
    const int g = P.gsrch;
    const int BIG = 1 << 30;

    // The warp's lanes are searched in groups: a group is the lanes whose cell is the first
    // remaining lane's cell or the next cell of its row (the lanes' cells ascend with the
    // lane index).  In dense regions a warp is one or two such cells and this is one pass; in
    // sparse regions a warp's particles can come from distant cells, and searching them
    // apart keeps each box and window small.  Within a group the search is unchanged.
    uint32_t n = 0;
    unsigned remaining = __ballot_sync(0xffffffffu, act);
    while (remaining) {
        const int leader = __ffs(remaining) - 1;
        const uint32_t lcell = __shfl_sync(0xffffffffu, pcell, leader);
        // group: the lanes whose cell is the leader's cell or (group mode 0) the next cell of its
        // row (any lanes may share a search: each takes its own window cells in ascending
        // index, its adjacency order; the rule only keeps the group's box compact)
        // (the next cell is in the leader's row unless the leader's cell ends the row: x = res - 1)
        const uint32_t span = P.group_mode == 0 ? 1u : 0u;
        const bool row_next = __shfl_sync(0xffffffffu, win.x, leader) + 2 < P.res[0];
        const bool ing = act && ((remaining >> lane) & 1u) && pcell >= lcell && pcell - lcell <= span &&
                         (pcell == lcell || row_next);
        remaining &= ~__ballot_sync(0xffffffffu, ing);
        // the group's particles span [t?0, t?1]; the search box is that span widened by Rf
        const float tx0 = warp_min(ing ? ip.x : INF), tx1 = warp_max(ing ? ip.x : -INF);
        const float ty0 = warp_min(ing ? ip.y : INF), ty1 = warp_max(ing ? ip.y : -INF);
        const float tz0 = warp_min(ing ? ip.z : INF), tz1 = warp_max(ing ? ip.z : -INF);
        const int wx0 = warp_mini(ing ? win.x : BIG), wx1 = warp_maxi(ing ? win.x : -BIG) + g - 1;
        const int wy0 = warp_mini(ing ? win.y : BIG), wy1 = warp_maxi(ing ? win.y : -BIG) + g - 1;
        const int wz0 = warp_mini(ing ? win.z : BIG), wz1 = warp_maxi(ing ? win.z : -BIG) + g - 1;
        // The group's window cells, in ascending linear index (y, then z, then x), are looked
        // up 32 at a time, one per lane, skipping cells whose box misses the group's box; the
        // non-empty ones are then taken in order.
        const int ncx = wx1 - wx0 + 1, ncz = wz1 - wz0 + 1;
        const int ncell = ncx * ncz * (wy1 - wy0 + 1);
        // packed instances: the group's instance, whose frame places its cells (a group's cells
        // belong to one instance)
        const uint32_t ginst = PACKED ? X.iid[__shfl_sync(0xffffffffu, p, leader)] : UNDEF;
        for (int cb = 0; cb < ncell; cb += 32) {
            const int t = cb + (int)lane;
            uint32_t tcnt = 0, toff = 0, tpos = 0;  // tpos: the cell's offsets in the window
            if (t < ncell) {
                const int ox = t % ncx, oz = (t / ncx) % ncz, oy = t / (ncx * ncz);
                tpos = (uint32_t)ox | ((uint32_t)oy << 8) | ((uint32_t)oz << 16);
                const int cx = wx0 + ox, cz = wz0 + oz, cy = wy0 + oy;
                if (!prune || cell_meets_box(PACKED ? frame_of(P, ginst) : frame_of(P), cx, cy, cz,
                                             tx0 - Rf, tx1 + Rf, ty0 - Rf, ty1 + Rf, tz0 - Rf, tz1 + Rf)) {
                    const uint32_t cell = checked(P, (uint32_t)((cy * P.res[2] + cz) * P.res[0] + cx), P.cells);
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
                uint32_t mark = LIST_CELL_START;  // flags a lane's first neighbour in this cell
                for (uint32_t base = 0; base < cnt; base += 32) {
                    const uint32_t kk = base + lane;
                    const bool valid = kk < cnt;
                    const float4 qp = valid ? pos[checked(P, off + kk, P.cap)] : make_float4(INF, INF, INF, 0.f);
                    // survivors: candidates within Rf of the span (the span's box with rounded
                    // edges and corners); every lane's neighbour is one, as the lane lies in it
                    const float ex = fmaxf(0.f, fmaxf(tx0 - qp.x, qp.x - tx1));
                    const float ey = fmaxf(0.f, fmaxf(ty0 - qp.y, qp.y - ty1));
                    const float ez = fmaxf(0.f, fmaxf(tz0 - qp.z, qp.z - tz1));
                    const bool surv = valid && ex * ex + ey * ey + ez * ez <= Rf * Rf;
                    const unsigned ball = __ballot_sync(0xffffffffu, surv);
                    if (surv) {
                        const uint32_t slot = (uint32_t)__popc(ball & ((1u << lane) - 1u));
                        s_sx[w][slot] = qp.x;
                        s_sy[w][slot] = qp.y;
                        s_sz[w][slot] = qp.z;
                        s_sq[w][slot] = off + kk;
                    }
                    __syncwarp();
                    const int ns = __popc(ball);
                    if (inw) {
                        // Membership uses a fused-multiply-add distance with a slack of a few
                        // ulps, so the list is a superset of the neighbours; the exact test is
                        // made again when the list is evaluated.  Four survivors per iteration,
                        // their distances two at a time in packed f32x2 operations (the same
                        // fused expression per component as approx_dsq: list membership only);
                        // a hit is written at the lane's next free row by a predicated store
                        // (no divergent branch, no shared-memory store for the misses; a full
                        // list writes to a spare row).
                        const float2 m1 = make_float2(-1.f, -1.f);
                        const float2 px = make_float2(ip.x, ip.x), py = make_float2(ip.y, ip.y),
                                     pz = make_float2(ip.z, ip.z);
                        int tt = 0;
                        for (; tt + 4 <= ns; tt += 4) {
                            const float4 X = *reinterpret_cast<const float4*>(&s_sx[w][tt]);
                            const float4 Y = *reinterpret_cast<const float4*>(&s_sy[w][tt]);
                            const float4 Z = *reinterpret_cast<const float4*>(&s_sz[w][tt]);
                            const uint4 Q = *reinterpret_cast<const uint4*>(&s_sq[w][tt]);
                            float2 dx = __ffma2_rn(make_float2(X.x, X.y), m1, px);
                            float2 dy = __ffma2_rn(make_float2(Y.x, Y.y), m1, py);
                            float2 dz = __ffma2_rn(make_float2(Z.x, Z.y), m1, pz);
                            const float2 d01 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                            dx = __ffma2_rn(make_float2(X.z, X.w), m1, px);
                            dy = __ffma2_rn(make_float2(Y.z, Y.w), m1, py);
                            dz = __ffma2_rn(make_float2(Z.z, Z.w), m1, pz);
                            const float2 d23 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                            const float d[4] = {d01.x, d01.y, d23.x, d23.y};
                            const uint32_t qi[4] = {Q.x, Q.y, Q.z, Q.w};
                            // the batch's row pointer advances by a row per hit; the hits are
                            // counted from it once per batch
                            uint32_t* const wp0 = my + min(n, (uint32_t)NL_CAP) * 32;
                            uint32_t* wp = wp0;
#pragma unroll
                            for (int u = 0; u < 4; u++) {
                                const bool hit = d[u] < R2s && d[u] > 0.f;
                                if (hit) *wp = qi[u] | mark;
                                mark = hit ? 0u : mark;
                                wp += hit ? 32 : 0;
                            }
                            n += (uint32_t)(wp - wp0) >> 5;
                        }
                        for (; tt < ns; tt++) {
                            const float4 sp = make_float4(s_sx[w][tt], s_sy[w][tt], s_sz[w][tt], 0.f);
                            const float d = approx_dsq(ip, sp);
                            const bool hit = d < R2s && d > 0.f;
                            if (hit) my[min(n, (uint32_t)NL_CAP) * 32] = s_sq[w][tt] | mark;
                            mark = hit ? 0u : mark;
                            n += hit ? 1u : 0u;
                        }
                    }
                    __syncwarp();
                }
            }
        }
    }
    const bool over = act && n > (uint32_t)NL_CAP;
    if (act && !over) {
        if (PACKED)  // the particle's own genome
            dens_list_finish<FLAGS>(P, P.genomes + X.iid[p], p, ip, n, my, pos, conc_in, conc_out, genes,
                                    press, invdens, flist, fcount, X, k);
        else
            dens_list_finish<FLAGS>(P, G, p, ip, n, my, pos, conc_in, conc_out, genes, press, invdens,
                                    flist, fcount, X, k);
    }
    // Lanes with more neighbours than the list holds (dense clumps): the warp takes them one at a
    // time with the overflow walk, its list rows (read by now) holding the segments' hits.
    unsigned ob = __ballot_sync(0xffffffffu, over);
    if (!ob) return;
    __syncwarp();
    uint8_t* const scratch = reinterpret_cast<uint8_t*>(s_list + (size_t)w * NL_ROWS * 32);
    float4 (*const o_cj)[NTF / 4] = reinterpret_cast<float4 (*)[NTF / 4]>(scratch);
    float* const o_d = reinterpret_cast<float*>(scratch + OVF_SEG * NTF * sizeof(float));
    uint32_t* const o_q = reinterpret_cast<uint32_t*>(scratch + OVF_SEG * (NTF + 1) * sizeof(float));
    uint8_t* const o_c = scratch + OVF_SEG * (NTF + 2) * sizeof(float);
    while (ob) {
        const int src = __ffs(ob) - 1;
        ob &= ob - 1;
        ovf_particle<FLAGS, PACKED>(P, G, __shfl_sync(0xffffffffu, p, src), pos, conc_in, conc_out, genes,
                                    scell, count, offset, press, invdens, flist, fcount, X, prune, o_cj,
                                    o_d, o_q, o_c);
    }
    if (over && X.hlist) X.hcount[k] = UNDEF;  // the re-forming search walks its cells again
}

// ---- per-lane fine-cell search ----------------------------------------------------------------
// For search radii up to half a grid cell.  The processing order groups each cell's particles
// by 2x2x2 sub-cell (sub_bits 1) and the cell sort records each cell's eight sub-cell counts, so
// every lane walks only the sub-cells within its radius: the fine cells floor(2g - rf) ..
// floor(2g + rf) per axis (g the particle's cell coordinate, rf the radius in fine cells with a
// margin for the rounding of g), grouped by grid cell in ascending cell index.  Hits of one
// cell are kept in ascending sorted index by insertion, so the list has the canonical order.
template <int FLAGS>
__global__ void __launch_bounds__(DENS_WARPS * 32, MG_DENS_MIN_BLOCKS) k_dens_fine(
    DevParams P, const DevGenome* __restrict__ G, const float4* __restrict__ pos,
    const float* __restrict__ conc_in, float* __restrict__ conc_out,
    const uint32_t* __restrict__ genes, const uint32_t* __restrict__ scell,
    const uint32_t* __restrict__ count, const uint32_t* __restrict__ offset,
    const unsigned long long* __restrict__ subcnt, float* __restrict__ press,
    float* __restrict__ invdens, uint32_t* __restrict__ flist, uint32_t* __restrict__ fcount,
    const uint32_t* __restrict__ nactive_p, const uint32_t* __restrict__ work,
    uint32_t* __restrict__ ovf, uint32_t* __restrict__ ovf_count, DensExtra X) {
    using F = DF<FLAGS>;
    extern __shared__ uint32_t s_list[];  // [warps of the block][NL_CAP][32]
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t* my = s_list + (size_t)w * NL_CAP * 32 + lane;
    const uint32_t k0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 >= *nactive_p) {
        park_conc<FLAGS>(conc_in, conc_out, k0, *nactive_p, P.cap);
        return;
    }
    const uint32_t p = work[k0];
    const float4 ip = pos[p];
    float R2 = 1.f;
    if (F::DENS) R2 = fmaxf(R2, P.r2);
    if (F::DIFF || F::MEAN) R2 = fmaxf(R2, P.r2diff);
    const float R2s = R2 * 1.000004f;  // list threshold for the fused distance (superset)
    const float Rw = sqrtf(R2);
    // fine-cell range per axis, clipped to the 27-cell window of the particle's own cell
    int lo[3], hi[3];
    {
        const float c[3] = {ip.x, ip.y, ip.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float g = (c[a] - P.gmin[a]) * P.gdelta[a];
            const int own = (int)g;  // the cell hash of the insert pass
            const float g2 = 2.f * g;
            const float rf = 2.f * Rw * P.gdelta[a] * 1.0002f + 1e-3f;
            lo[a] = max((int)floorf(g2 - rf), 2 * (own - 1));
            hi[a] = min((int)floorf(g2 + rf), 2 * (own + 1) + 1);
        }
    }
    uint32_t n = 0;
    for (int cy = lo[1] >> 1; cy <= (hi[1] >> 1); cy++) {
        for (int cz = lo[2] >> 1; cz <= (hi[2] >> 1); cz++) {
            for (int cx = lo[0] >> 1; cx <= (hi[0] >> 1); cx++) {
                const uint32_t cell = (uint32_t)((cy * P.res[2] + cz) * P.res[0] + cx);
                const uint32_t cnt = count[cell];
                if (cnt == 0) continue;
                const uint32_t off = offset[cell];
                const uint32_t seg = n;  // this cell's hits start here
                // sub-cell ranges of this cell inside the fine window
                const int sx0 = max(lo[0] - 2 * cx, 0), sx1 = min(hi[0] - 2 * cx, 1);
                const int sy0 = max(lo[1] - 2 * cy, 0), sy1 = min(hi[1] - 2 * cy, 1);
                const int sz0 = max(lo[2] - 2 * cz, 0), sz1 = min(hi[2] - 2 * cz, 1);
                uint32_t starts[9];
                const bool whole = cnt >= (uint32_t)WARP_CELL_MAX;  // no sub-cell counts: scan it all
                if (!whole) {
                    const unsigned long long sc = subcnt[cell];
                    uint32_t acc = 0;
#pragma unroll
                    for (int code = 0; code < 8; code++) {
                        starts[code] = acc;
                        acc += (uint32_t)((sc >> (8 * code)) & 0xFFu);
                    }
                    starts[8] = acc;
                }
                for (int sz = whole ? 0 : sz0; sz <= (whole ? 0 : sz1); sz++)
                    for (int sy = whole ? 0 : sy0; sy <= (whole ? 0 : sy1); sy++)
                        for (int sx = whole ? 0 : sx0; sx <= (whole ? 0 : sx1); sx++) {
                            const int code = sx | (sy << 1) | (sz << 2);
                            const uint32_t b = whole ? 0u : starts[code];
                            const uint32_t e = whole ? cnt : starts[code + 1];
                            for (uint32_t t = b; t < e; t++) {
                                const uint32_t q = work[off + t];
                                const float d = approx_dsq(ip, pos[q]);
                                if (!(d < R2s && d > 0.f)) continue;
                                if (n < (uint32_t)NL_CAP) {  // insert in ascending index
                                    uint32_t i = n;
                                    while (i > seg && my[(i - 1) * 32] > q) {
                                        my[i * 32] = my[(i - 1) * 32];
                                        i--;
                                    }
                                    my[i * 32] = q;
                                }
                                n++;
                            }
                        }
                if (n > seg && seg < (uint32_t)NL_CAP) my[seg * 32] |= LIST_CELL_START;
            }
        }
    }
    if (n > (uint32_t)NL_CAP) {
        ovf[atomicAdd(ovf_count, 1u)] = p;
        if (X.hlist) X.hcount[k0] = UNDEF;
        return;
    }
    dens_list_finish<FLAGS>(P, G, p, ip, n, my, pos, conc_in, conc_out, genes, press, invdens, flist,
                            fcount, X, k0);
}

template <int FLAGS, bool PACKED = false>
__global__ void __launch_bounds__(256, 1) k_dens_ovf(
    DevParams P, const DevGenome* __restrict__ G0, const float4* __restrict__ pos,
    const float* __restrict__ conc_in, float* __restrict__ conc_out,
    const uint32_t* __restrict__ genes, const uint32_t* __restrict__ scell,
    const uint32_t* __restrict__ count, const uint32_t* __restrict__ offset,
    float* __restrict__ press, float* __restrict__ invdens, uint32_t* __restrict__ flist,
    uint32_t* __restrict__ fcount, const uint32_t* __restrict__ ovf,
    const uint32_t* __restrict__ ovf_count, DensExtra X, bool prune) {
    __shared__ float4 s_cj[256 / 32][OVF_SEG][NTF / 4];  // concentrations of the segment's hits
    __shared__ float s_d[256 / 32][OVF_SEG];
    __shared__ uint32_t s_q[256 / 32][OVF_SEG];
    __shared__ uint8_t s_c[256 / 32][OVF_SEG];
    const uint32_t wl = threadIdx.x >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    uint32_t nq = *ovf_count;
    if (nq > P.cap) nq = P.cap;
    for (uint32_t e = gw; e < nq; e += nw)
        ovf_particle<FLAGS, PACKED>(P, G0, ovf[e], pos, conc_in, conc_out, genes, scell, count, offset,
                                    press, invdens, flist, fcount, X, prune, s_cj[wl], s_d[wl], s_q[wl],
                                    s_c[wl]);
}

// The per-lane lists take 48 KB of dynamic shared memory next to the static survivor buffers,
// above the 48 KB a launch gets without opting in.
#define MG_DENS_FLAG_SETS(M) M(1) M(2) M(3) M(5) M(6) M(7) M(9) M(23) M(46) M(47)
// the flag sets of packed instances (physics and the plain morphogen stage)
#define MG_DENS_PACKED_SETS(M) M(1) M(2) M(3) M(5) M(6) M(7)

cudaError_t physics_init() {
    const int smem = DENS_WARPS * NL_ROWS * 32 * (int)sizeof(uint32_t);
    cudaError_t e = cudaSuccess;
#define MG_ATTR(F)                                                                              \
    if (e == cudaSuccess)                                                                       \
        e = cudaFuncSetAttribute(k_dens_warp<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
    if (e == cudaSuccess)                                                                       \
        e = cudaFuncSetAttribute(k_dens_fine<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    MG_DENS_FLAG_SETS(MG_ATTR)
#undef MG_ATTR
#define MG_ATTR_PACKED(F)                                                                       \
    if (e == cudaSuccess)                                                                       \
        e = cudaFuncSetAttribute(k_dens_warp<F, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    MG_DENS_PACKED_SETS(MG_ATTR_PACKED)
#undef MG_ATTR_PACKED
    return e;
}

void launch_dens(const DevParams& P, const DevGenome* G, const DevGenome& Gh, const Carried& cur, const float* conc_in,
                 float* conc_out, const Scratch& s, int flags, int search, int num_sms,
                 cudaStream_t st, const DensExtra* extra) {
    DensExtra X = extra ? *extra : DensExtra{};
    X.epi = P.full_epi ? cur.epi : nullptr;
    X.iid = cur.iid;
    const int warps = (P.dens_warps >= 1 && P.dens_warps <= DENS_WARPS) ? P.dens_warps : DENS_WARPS;
    const size_t smem = (size_t)warps * NL_ROWS * 32 * sizeof(uint32_t);
    if ((search == 1 || search == 3) && (flags & (1 | 2 | 8 | 16))) {
        uint32_t blocks = (P.cap + warps * 32 - 1) / (warps * 32);
        const bool prune = search == 1;
#define MG_DENSW_CASE_P(F, PK)                                                                    \
    case F:                                                                                       \
        k_dens_warp<F, PK><<<blocks, warps * 32, smem, st>>>(P, MG_DENS_GENOME_ARG, cur.pos, conc_in, conc_out, \
                                                             cur.genes, s.scell, s.count,         \
                                                             s.offset, cur.press, cur.invdens,        \
                                                             s.flist, s.fcount, s.counters + 3,   \
                                                             s.work, X, prune);                   \
        return;
#define MG_DENSW_CASE(F) MG_DENSW_CASE_P(F, false)
#define MG_DENSW_CASE_PACKED(F) MG_DENSW_CASE_P(F, true)
        if (cur.iid) {
            switch (flags) { MG_DENS_PACKED_SETS(MG_DENSW_CASE_PACKED) default: break; }
        } else {
            switch (flags) { MG_DENS_FLAG_SETS(MG_DENSW_CASE) default: break; }
        }
#undef MG_DENSW_CASE
#undef MG_DENSW_CASE_PACKED
#undef MG_DENSW_CASE_P
    }
    if (search == 2 && (flags & (1 | 2 | 8 | 16))) {
        uint32_t blocks = (P.cap + warps * 32 - 1) / (warps * 32);
#define MG_DENSF_CASE(F)                                                                          \
    case F:                                                                                       \
        k_dens_fine<F><<<blocks, warps * 32, smem, st>>>(P, G, cur.pos, conc_in, conc_out,        \
                                                         cur.genes, s.scell, s.count, s.offset,   \
                                                         s.subcnt, cur.press, cur.invdens, s.flist,   \
                                                         s.fcount, s.counters + 3, s.work, s.ovf, \
                                                         s.counters + 6, X);                      \
        k_dens_ovf<F><<<(uint32_t)num_sms * 4, 256, 0, st>>>(P, G, cur.pos, conc_in, conc_out,    \
                                                             cur.genes, s.scell, s.count,         \
                                                             s.offset, cur.press, cur.invdens,        \
                                                             s.flist, s.fcount, s.ovf,            \
                                                             s.counters + 6, X, true);            \
        return;
        cudaMemsetAsync(s.counters + 6, 0, sizeof(uint32_t), st);
        switch (flags) { MG_DENS_FLAG_SETS(MG_DENSF_CASE) default: break; }
#undef MG_DENSF_CASE
    }
    uint32_t blocks = (P.cap + 255) / 256;
#define MG_DENS_CASE(F)                                                                        \
    case F:                                                                                    \
        k_dens<F><<<blocks, 256, 0, st>>>(P, G, cur.pos, conc_in, conc_out, cur.genes, s.scell, \
                                          s.count, s.offset, cur.press, cur.invdens,              \
                                          s.counters + 3, X);                                  \
        return;
    switch (flags) { MG_DENS_FLAG_SETS(MG_DENS_CASE) MG_DENS_CASE(4) default: break; }
#undef MG_DENS_CASE
}

// ---- force -------------------------------------------------------------------------------
// computeForce skips a bond when `restlength < 0.000000001` with the float promoted to double
// (cuda:3268).  For every float x that test equals x < REST_MIN, REST_MIN being the smallest
// float not below 1e-9 (0x30897060 = 1.0000000604e-9), so it runs on the FP32 pipe.
#define REST_MIN __int_as_float(0x30897060)
// Elastic bond term of bond (owner o -> partner j) as computeForce evaluates it in the owner's
// thread (cuda:3263-3307).  Returns the acceleration pushed onto the partner; the owner
// subtracts it.
struct BondTerm {
    float ex, ey, ez, strain, absd;
};

__device__ __forceinline__ BondTerm bond_term(float4 po, float4 vo, float4 pj, float4 vj,
                                              float restlen, float modulus, float damping,
                                              float elastlim, float pmass) {
    BondTerm t;
    const float dx = po.x - pj.x, dy = po.y - pj.y, dz = po.z - pj.z;
    const float dsq = dx * dx + dy * dy + dz * dz;
    const float absd = sqrtf(dsq) + FLT_MIN;
    const float rvx = vj.x - vo.x, rvy = vj.y - vo.y, rvz = vj.z - vo.z;
    const float q = (absd - restlen) / restlen;
    const float strain = q > 0.f ? q : 0.f;  // fmaxf(0, q), NaN -> 0
    const float flag = (float)(absd < elastlim);
    t.ex = (flag * (((dx / absd) * strain) * modulus - damping * rvx)) / pmass;
    t.ey = (flag * (((dy / absd) * strain) * modulus - damping * rvy)) / pmass;
    t.ez = (flag * (((dz / absd) * strain) * modulus - damping * rvz)) / pmass;
    t.strain = strain;
    t.absd = absd;
    return t;
}

__device__ __forceinline__ bool is_nan3(const BondTerm& t) {
    return t.ex != t.ex || t.ey != t.ey || t.ez != t.ez;
}

// Fluid pressure, surface and viscosity terms of one neighbour (contributeForce, cuda:3203-3221).
__device__ __forceinline__ void fluid_term(const DevParams& P, float4 ip, float4 iv, float ipress,
                                           float idens, float4 jp, float4 jv, float jpress,
                                           float jdens, float dsq, float dx, float dy, float dz,
                                           float& cx, float& cy, float& cz) {
    const float r = sqrtf(dsq);
    const float t = P.sr - r;
    const float kern = t * t * t;
    const float prs = 100.f * (ipress + jpress);
    const float s = (idens * jdens) * 100.f;
    const float term = prs * kern - P.surf * (t * t);
    const float px = (s * (dx / r)) * term, py = (s * (dy / r)) * term, pz = (s * (dz / r)) * term;
    const float vx = (100000.f * (jv.x - iv.x)) * kern;
    const float vy = (100000.f * (jv.y - iv.y)) * kern;
    const float vz = (100000.f * (jv.z - iv.z)) * kern;
    cx = cx + (px + vx);
    cy = cy + (py + vy);
    cz = cz + (pz + vz);
}

__global__ void __launch_bounds__(MG_PLAIN_MAX_THREADS) k_force(DevParams P, Carried C,
                                               const uint32_t* __restrict__ scell,
                                               const uint32_t* __restrict__ count,
                                               const uint32_t* __restrict__ offset,
                                               const float* __restrict__ press,
                                               const float* __restrict__ invdens,
                                               const uint32_t* __restrict__ flist,
                                               const uint32_t* __restrict__ fcount, int use_list,
                                               float4* __restrict__ force,
                                               float4* __restrict__ bterm,
                                               uint32_t* __restrict__ brk,
                                               const uint32_t* __restrict__ nactive_p) {
    // First of the two force kernels: own bonds and fluid terms.  Each own bond's acceleration
    // on its partner goes to bterm, where the second kernel gathers the partner's incoming
    // reactions once every owner has written them.
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nact = *nactive_p;
    if (p >= nact) return;
    const uint32_t cap = P.cap;
    const float4 ip = C.pos[p], iv = C.veval[p];
    // the bond records' slot; a particle without an origin (a slot that was parked and given a
    // position again by an upload) has no bonds
    const uint32_t o0 = C.origin[p] == UNDEF ? UNDEF : checked(P, C.origin[p], cap);
    const bool has_rec = o0 != UNDEF;
    const uint32_t o = has_rec ? o0 : 0u;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    uint32_t br = 0;
    // own (outgoing) bonds
#pragma unroll
    for (int a = 0; a < NB; a++) {
        uint4* recb = C.bond + bond_ib(cap, a, o);
        const uint4 A = C.bond[bond_ia(cap, a, o)], B = *recb;
        const uint32_t j = has_rec ? C.partner[bond_ip(cap, a, o)] : NO_PARTNER;
        const float restlen = __uint_as_float(A.y);
        if (j >= nact || restlen < REST_MIN) {
            bterm[(size_t)a * cap + p] = make_float4(0.f, 0.f, 0.f, __uint_as_float(UNDEF));
            continue;
        }
        const float elastlim = __uint_as_float(B.x);
        const BondTerm t = bond_term(ip, iv, C.pos[j], C.veval[j], restlen, __uint_as_float(A.z),
                                     __uint_as_float(A.w), elastlim, P.pmass);
        const float sq = __uint_as_float(B.z) + t.strain * t.strain;
        const float si = __uint_as_float(B.w) + t.strain;
        *reinterpret_cast<uint2*>(&recb->z) = make_uint2(__float_as_uint(sq), __float_as_uint(si));
        bterm[(size_t)a * cap + p] = make_float4(t.ex, t.ey, t.ez, __uint_as_float(j));
        if (!is_nan3(t)) {
            fx = fx - t.ex;
            fy = fy - t.ey;
            fz = fz - t.ez;
        }
        if (t.absd >= elastlim && !P.freeze) br |= 1u << a;
    }
    // fluid pressure, surface and viscosity terms (contributeForce, cuda:3167-3226)
    {
        const float ipress = press[p], idens = invdens[p];
        float sx = 0.f, sy = 0.f, sz = 0.f;
        const uint32_t nf = use_list ? fcount[p] : 0xFFFFFFFFu;
        if (nf <= (uint32_t)FL_CAP) {
            float cx = 0.f, cy = 0.f, cz = 0.f;
            // One neighbour's term; its list entry flags the first neighbour of each cell,
            // where the previous cell's partial sum is flushed.
            auto term = [&](uint32_t e, float4 jp, float4 jv, float jpress, float jdens) {
                if (e & FLIST_CELL_START) {
                    sx = sx + cx; sy = sy + cy; sz = sz + cz;
                    cx = cy = cz = 0.f;
                }
                const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
                const float dsq = dx * dx + dy * dy + dz * dz;
                fluid_term(P, ip, iv, ipress, idens, jp, jv, jpress, jdens, dsq, dx, dy, dz, cx, cy, cz);
            };
            uint32_t k = 0;
            // two neighbours per iteration, so their gathers are in flight together, and the
            // next two list entries loaded one iteration ahead
            uint32_t e0n = nf >= 2 ? flist[p] : 0u, e1n = nf >= 2 ? flist[(size_t)cap + p] : 0u;
            for (; k + 2 <= nf; k += 2) {
                const uint32_t e0 = e0n, e1 = e1n;
                if (k + 4 <= nf) {
                    e0n = flist[(size_t)(k + 2) * cap + p];
                    e1n = flist[(size_t)(k + 3) * cap + p];
                }
                const uint32_t q0 = checked(P, e0 & ~FLIST_CELL_START, cap), q1 = checked(P, e1 & ~FLIST_CELL_START, cap);
                const float4 jp0 = C.pos[q0], jp1 = C.pos[q1], jv0 = C.veval[q0], jv1 = C.veval[q1];
                const float pr0 = press[q0], pr1 = press[q1], dn0 = invdens[q0], dn1 = invdens[q1];
                term(e0, jp0, jv0, pr0, dn0);
                term(e1, jp1, jv1, pr1, dn1);
            }
            if (k < nf) {
                const uint32_t e = flist[(size_t)k * cap + p], q = checked(P, e & ~FLIST_CELL_START, cap);
                term(e, C.pos[q], C.veval[q], press[q], invdens[q]);
            }
            sx = sx + cx; sy = sy + cy; sz = sz + cz;
        } else {
            const uint32_t base = scell[p] - (uint32_t)P.nadj;
            for (int c = 0; c < P.adjcnt; c++) {
                const uint32_t cellc = base + (uint32_t)P.adj[c];
                const uint32_t cnt = count[cellc];
                if (cnt == 0) continue;
                const uint32_t off = offset[cellc];
                float cx = 0.f, cy = 0.f, cz = 0.f;
                for (uint32_t q = off; q < off + cnt; q++) {
                    const float4 jp = C.pos[q];
                    const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
                    const float dsq = dx * dx + dy * dy + dz * dz;
                    if (dsq < 1.f && dsq > 0.f)
                        fluid_term(P, ip, iv, ipress, idens, jp, C.veval[q], press[q], invdens[q], dsq,
                                   dx, dy, dz, cx, cy, cz);
                }
                sx = sx + cx; sy = sy + cy; sz = sz + cz;
            }
        }
        fx = fx + sx * P.pmass;
        fy = fy + sy * P.pmass;
        fz = fz + sz * P.pmass;
    }
    force[p] = make_float4(fx, fy, fz, 0.f);
    brk[p] = br;
}

// Second force kernel: the reactions of incoming bonds, in slot order (the gather form of the
// atomicAdd at cuda:3311-3313), added to the first kernel's sum.  An owner's stored term is the
// one its own-bond loop evaluated for this particle as partner: the same arguments, the same
// bits as evaluating it here.  Run by k_force_in, or at the top of the integration when it
// follows the force pass directly.
__device__ __forceinline__ float4 add_incoming(uint32_t cap, const uint32_t* __restrict__ pidx,
                                               const float4* __restrict__ bterm,
                                               const float4* __restrict__ force, uint32_t p, uint32_t nact) {
    const uint4* pi = reinterpret_cast<const uint4*>(pidx + (size_t)p * 12);
    uint32_t in[12];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint4 v = pi[k];
        in[4 * k] = v.x; in[4 * k + 1] = v.y; in[4 * k + 2] = v.z; in[4 * k + 3] = v.w;
    }
    float4 t[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) {  // all gathers in flight before the sums
        const uint32_t k = in[2 * b], bk = in[2 * b + 1];
        t[b] = (k < nact && bk < (uint32_t)NB) ? bterm[(size_t)bk * cap + k]
                                                 : make_float4(0.f, 0.f, 0.f, __uint_as_float(UNDEF));
    }
    float4 f = force[p];
#pragma unroll
    for (int b = 0; b < NB; b++) {
        if (__float_as_uint(t[b].w) != p) continue;  // the owner's slot no longer bonds to p
        if (t[b].x != t[b].x || t[b].y != t[b].y || t[b].z != t[b].z) continue;
        f.x = f.x + t[b].x;
        f.y = f.y + t[b].y;
        f.z = f.z + t[b].z;
    }
    return f;
}

__global__ void __launch_bounds__(MG_PLAIN_MAX_THREADS) k_force_in(uint32_t cap, const uint32_t* __restrict__ pidx,
                                                  const float4* __restrict__ bterm,
                                                  float4* __restrict__ force,
                                                  const uint32_t* __restrict__ nactive_p) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nact = *nactive_p;
    if (p >= nact) return;
    force[p] = add_incoming(cap, pidx, bterm, force, p, nact);
}

void launch_force(const DevParams& P, const Carried& cur, const Scratch& s, bool use_list,
                  cudaStream_t st, bool incoming_in_advance) {
    const uint32_t nt = (uint32_t)P.force_threads, blocks = (P.cap + nt - 1) / nt;
    k_force<<<blocks, nt, 0, st>>>(P, cur, s.scell, s.count, s.offset, cur.press, cur.invdens, s.flist,
                                    s.fcount, use_list ? 1 : 0, s.force, s.bterm, s.brk, s.counters + 3);
    if (!incoming_in_advance) k_force_in<<<blocks, nt, 0, st>>>(P.cap, cur.pidx, s.bterm, s.force, s.counters + 3);
}

// Broken bonds get rest length 0 (cuda:3315-3317).  The force kernel records the breaks in
// brk[] instead of writing the rest length, because other threads of the same kernel read
// that rest length for their incoming-bond reactions.
// Rest length 0 on the bonds that broke (o: the particle's origin, where its records live).
__device__ __forceinline__ void apply_breaks(uint4* bond, uint32_t cap, uint32_t o, uint32_t br) {
#pragma unroll
    for (int a = 0; a < NB; a++)
        if (br & (1u << a)) reinterpret_cast<uint32_t*>(bond + bond_ia(cap, a, o))[1] = 0u;
}

__global__ void __launch_bounds__(256) k_apply_breaks(uint32_t cap, uint4* __restrict__ bond,
                                                      const uint32_t* __restrict__ origin,
                                                      const uint32_t* __restrict__ brk,
                                                      const uint32_t* __restrict__ nactive_p) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p) return;
    const uint32_t br = brk[p], o = origin[p];
    if (br && o != UNDEF) apply_breaks(bond, cap, o, br);
}

void launch_apply_breaks(const DevParams& P, const Carried& cur, const Scratch& s, cudaStream_t st) {
    uint32_t blocks = (P.cap + 255) / 256;
    k_apply_breaks<<<blocks, 256, 0, st>>>(P.cap, cur.bond, cur.origin, s.brk, s.counters + 3);
}

// ---- advance -----------------------------------------------------------------------------
__device__ __forceinline__ void wall(float& ax, float& ay, float& az, float diff, float nx,
                                     float ny, float nz, float stiff, float damp, float4 ve) {
    if (diff > 0.00001f) {  // EPSILON, fluid_system_cuda.cuh:41
        const float adj = stiff * diff - damp * (nx * ve.x + ny * ve.y + nz * ve.z);
        ax = ax + nx * adj;
        ay = ay + ny * adj;
        az = az + nz * adj;
    }
}

// sin(x) by Cody-Waite reduction to [-pi/4, pi/4] (pi/2 split in three floats, the first two
// with 12 significant bits so k * part is exact for |k| < 2^12) and Taylor polynomials of degree
// 9 (sine) and 8 (cosine); written as separate multiplies and adds so the oracle's C copy gives
// the same bits.
__device__ __forceinline__ float mg_sin_cw(float x) {
    const float P1 = 1.5703125f, P2 = __int_as_float(0x39fda000), P3 = __int_as_float(0x33a22169);
    if (x - x != 0.0f) return x - x;  // NaN or infinity: NaN
    const float k = rintf(x * 0.636619772f);
    const float r = ((x - k * P1) - k * P2) - k * P3;
    const int q = (int)k & 3;
    const float s = r * r;
    const float sn = r + r * s * ((-1.0f / 6.0f) + s * ((1.0f / 120.0f) + s * ((-1.0f / 5040.0f) + s * (1.0f / 362880.0f))));
    const float cs = 1.0f + s * (-0.5f + s * ((1.0f / 24.0f) + s * ((-1.0f / 720.0f) + s * (1.0f / 40320.0f))));
    return q == 0 ? sn : q == 1 ? cs : q == 2 ? -sn : -cs;
}

// Device copy of the simulation time: two slots alternating with the step counter's parity
// (counters[5], advanced by the insert pass), so the advance pass reads this step's time and
// writes the next one without a race.
__device__ __forceinline__ float* time_slot(uint32_t* counters, uint32_t step) {
    return reinterpret_cast<float*>(counters + 7 + (step & 1u));
}

// IN: the force pass left the incoming-bond reactions to this kernel (k_force_in's sum, written
// back to the force buffer, then integrated).
template <bool APPLY_BRK, bool SPECIAL, bool IN>
__global__ void __launch_bounds__(MG_PLAIN_MAX_THREADS) k_advance(DevParams P, Carried C,
                                                 float4* __restrict__ force,
                                                 const float4* __restrict__ bterm,
                                                 const uint32_t* __restrict__ brk,
                                                 uint32_t* __restrict__ counters) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t step = counters[5];
    const float time = *time_slot(counters, step);
    if (p == 0) *time_slot(counters, step + 1u) = time + P.dt;  // AdvanceTime (fluid_system.cpp:2016)
    const uint32_t nact = counters[3];
    if (p >= nact) return;
    float4 f;
    if (IN) {
        f = add_incoming(P.cap, C.pidx, bterm, force, p, nact);
        force[p] = f;
    } else {
        f = force[p];
    }
    const float4 pos = C.pos[p], ve = C.veval[p];
    // the walls: the system's box, or a packed instance's own
    const float* bmin = C.iid ? P.inst[C.iid[p]].bmin : P.bmin;
    const float* bmax = C.iid ? P.inst[C.iid[p]].bmax : P.bmax;
    float ax = f.x, ay = f.y, az = f.z;
    float diff;
    diff = P.pr - (pos.y - (bmin[1] + (pos.x - bmin[0]) * P.slope));
    wall(ax, ay, az, diff, -P.slope, P.one_minus_slope, 0.f, P.estiff, P.damp, ve);
    diff = P.pr - (bmax[1] - pos.y);
    wall(ax, ay, az, diff, 0.f, -1.f, 0.f, P.estiff, P.damp, ve);
    diff = P.pr - (pos.x - bmin[0]);
    wall(ax, ay, az, diff, 1.f, 0.f, 0.f, P.xmin_stiff, P.damp, ve);
    diff = P.pr - (bmax[0] - pos.x);
    wall(ax, ay, az, diff, -1.f, 0.f, 0.f, P.xmax_stiff, P.damp, ve);
    diff = P.pr - (pos.z - bmin[2]);
    wall(ax, ay, az, diff, 0.f, 0.f, 1.f, P.estiff, P.damp, ve);
    diff = P.pr - (bmax[2] - pos.z);
    wall(ax, ay, az, diff, 0.f, 0.f, -1.f, P.estiff, P.damp, ve);
    {
        const float dx = bmax[0] - pos.x, dy = bmax[1] - pos.y, dz = bmax[2] - pos.z;
        diff = 2.f * P.pr - (dx + dy + dz);
        wall(ax, ay, az, diff, 1.f, 1.f, 1.f, P.estiff, P.damp, ve);
    }
    ax = ax + P.grav[0];
    ay = ay + P.grav[1];
    az = az + P.grav[2];
    float speed = ax * ax + ay * ay + az * az;
    if (speed > P.AL2) {
        const float s = P.AL / sqrtf(speed);
        ax *= s; ay *= s; az *= s;
    }
    float4 vel = C.vel[p];
    speed = vel.x * vel.x + vel.y * vel.y + vel.z * vel.z;
    if (speed > P.VL2) {  // speed = VL2; vel *= VL / sqrt(speed) (cuda:3576-3579)
        vel.x *= P.vl_factor; vel.y *= P.vl_factor; vel.z *= P.vl_factor;
    }
    const float dt = P.dt;
    const float vnx = ax * dt + vel.x, vny = ay * dt + vel.y, vnz = az * dt + vel.z;
    const uint32_t special = SPECIAL ? (C.genes[p] >> 11) & 3u : 0u;  // bit 0: gene 11, bit 1: gene 12
    if (special == 0) {
        C.veval[p] = make_float4((vel.x + vnx) * 0.5f, (vel.y + vny) * 0.5f, (vel.z + vnz) * 0.5f, ve.w);
        C.vel[p] = make_float4(vnx, vny, vnz, vel.w);
        C.pos[p] = make_float4(pos.x + vnx * dt, pos.y + vny * dt, pos.z + vnz * dt, pos.w);
    } else if (special == 2u) {
        // externalActuation (cuda:3617-3691): the previous state, z displaced by
        // actuation_factor * sin(time / (actuation_period * dt))
        const float ph = time / (P.actuation_period * dt);
        C.pos[p] = make_float4(pos.x, pos.y, pos.z + P.actuation_factor * mg_sin_cw(ph), pos.w);
    }
    // fixedParticles (cuda:3694-3705, after the actuation): the previous state is kept
    if (APPLY_BRK) {
        const uint32_t br = brk[p];
        if (br && C.origin[p] != UNDEF) apply_breaks(C.bond, P.cap, C.origin[p], br);
    }
}

template <bool APPLY_BRK, bool SPECIAL>
static void launch_advance_as(const DevParams& P, const Carried& cur, const Scratch& s, cudaStream_t st,
                              bool incoming) {
    const uint32_t nt = (uint32_t)P.advance_threads, blocks = (P.cap + nt - 1) / nt;
    if (incoming)
        k_advance<APPLY_BRK, SPECIAL, true><<<blocks, nt, 0, st>>>(P, cur, s.force, s.bterm, s.brk, s.counters);
    else
        k_advance<APPLY_BRK, SPECIAL, false><<<blocks, nt, 0, st>>>(P, cur, s.force, s.bterm, s.brk, s.counters);
}

void launch_advance(const DevParams& P, const Carried& cur, const Scratch& s, bool apply_brk,
                    cudaStream_t st, bool special, bool incoming) {
    if (apply_brk && special)
        launch_advance_as<true, true>(P, cur, s, st, incoming);
    else if (apply_brk)
        launch_advance_as<true, false>(P, cur, s, st, incoming);
    else if (special)
        launch_advance_as<false, true>(P, cur, s, st, incoming);
    else
        launch_advance_as<false, false>(P, cur, s, st, incoming);
}

}  // namespace mg
