// mg_physics.cu - SPH density/pressure, diffusion + gene reaction, bond + fluid force and
// leap-frog integration (rows a6-a10).  Compiled with -fmad=false: every kernel evaluates the
// float operations of the reference kernels in their order, without fused multiply-adds, so
// results are reproducible bit for bit against the CPU restatement.
//
// Reference: contributePressure/computePressure (fluid_system_cuda.cu:620-712),
// contributeDiffusion/computeDiffusion (cuda:3026-3105), computeGeneAction/tallyGeneAction
// (cuda:714-772), contributeForce/computeForce (cuda:3167-3358), advanceParticles
// (cuda:3470-3614).
#include <cfloat>
#include "mg_internal.cuh"

namespace mg {

// ---- density / pressure, diffusion, gene reaction ------------------------------------------
// One thread per sorted particle.  The neighbour loop visits the gridAdjCnt cells in the
// reference's gridAdj order and each cell's particles in sorted order; the density sum keeps
// the reference's per-cell partial sums.  FLAGS: 1 density/pressure, 2 diffusion,
// 4 gene reaction.  Diffusion reads conc_in for every neighbour and writes conc_out (Jacobi).
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
                                              const uint32_t* __restrict__ nactive_p) {
    constexpr bool DENS = FLAGS & 1, DIFF = FLAGS & 2, GENE = FLAGS & 4;
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p) return;
    const float4 ip = pos[p];
    float cur[NTF], nc[NTF], dif[NTF];
    if (DIFF || GENE) {
        const float4* c4 = reinterpret_cast<const float4*>(conc_in + (size_t)p * NTF);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            float4 v = c4[k];
            cur[4 * k] = v.x; cur[4 * k + 1] = v.y; cur[4 * k + 2] = v.z; cur[4 * k + 3] = v.w;
        }
    }
    if (DIFF) {
#pragma unroll
        for (int t = 0; t < NTF; t++) { nc[t] = 0.f; dif[t] = G->diff[t]; }
    }
    float sum = 0.f;
    if (DENS || DIFF) {
        const uint32_t base = scell[p] - (uint32_t)P.nadj;
        for (int c = 0; c < P.adjcnt; c++) {
            const uint32_t cellc = base + (uint32_t)P.adj[c];
            const uint32_t cnt = count[cellc];
            if (cnt == 0) continue;
            const uint32_t off = offset[cellc];
            float part = 0.f;
            for (uint32_t q = off; q < off + cnt; q++) {
                const float4 jp = pos[q];
                const float dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
                const float dsq = dx * dx + dy * dy + dz * dz;
                if (DENS && dsq < P.r2 && dsq > 0.f) {
                    const float r = sqrtf(dsq);
                    const float qq = r / P.sr;
                    float b = 1.f - qq;
                    b *= b;
                    b *= b;
                    part += b * (4.f * qq + 1.f);
                }
                if (DIFF && dsq < P.r2diff && dsq > 0.f) {
                    const float cc = (P.r2diff - dsq) * P.d2;
                    const float4* cj4 = reinterpret_cast<const float4*>(conc_in + (size_t)q * NTF);
                    float cj[NTF];
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        float4 v = cj4[k];
                        cj[4 * k] = v.x; cj[4 * k + 1] = v.y; cj[4 * k + 2] = v.z; cj[4 * k + 3] = v.w;
                    }
#pragma unroll
                    for (int t = 0; t < NTF; t++)
                        if (dif[t] != 0.f) nc[t] += (dif[t] * cc) * (cj[t] - cur[t]);
                }
            }
            if (DENS) sum += part;
        }
    }
    if (DENS) {
        sum = sum * P.pmass * P.wc2;
        if (sum == 0.f) sum = 1.f;
        press[p] = (sum - P.rest) * P.istiff;
        invdens[p] = 1.f / sum;
    }
    if (DIFF || GENE) {
        float c[NTF];
#pragma unroll
        for (int t = 0; t < NTF; t++) c[t] = DIFF ? G->breakdown[t] * (cur[t] + nc[t]) : cur[t];
        if (GENE) {
            // Gene bits are the sort-time dense-list membership (FEPIGEN > 0).  With every
            // FEPIGEN in {0, INT_MAX} and no activation lists the countdown never fires and
            // the reaction is: for each active gene g in order, activity = sum_tf sens*conc,
            // secretion accumulates rate*activity; living particles (gene 2) add it.
            const uint32_t bits = genes[p];
            float dc[NTF];
#pragma unroll
            for (int t = 0; t < NTF; t++) dc[t] = 0.f;
            for (int g = 0; g < NG; g++) {
                if (!((bits >> g) & 1u)) continue;
                float act = 0.f;
#pragma unroll
                for (int t = 0; t < NTF; t++) {
                    const float s = G->sens[g][t];
                    if (s != 0.f) act += s * c[t];
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
            if (bits & 4u) {
#pragma unroll
                for (int t = 0; t < NTF; t++) c[t] += dc[t];
            }
        }
        float4* o4 = reinterpret_cast<float4*>(conc_out + (size_t)p * NTF);
#pragma unroll
        for (int k = 0; k < 4; k++) o4[k] = make_float4(c[4 * k], c[4 * k + 1], c[4 * k + 2], c[4 * k + 3]);
    }
}

void launch_dens(const DevParams& P, const DevGenome* G, const Carried& cur, const float* conc_in,
                 float* conc_out, const Scratch& s, int flags, cudaStream_t st) {
    uint32_t blocks = (P.cap + 255) / 256;
#define MG_DENS_CASE(F)                                                                        \
    case F:                                                                                    \
        k_dens<F><<<blocks, 256, 0, st>>>(P, G, cur.pos, conc_in, conc_out, cur.genes, s.scell, \
                                          s.count, s.offset, s.press, s.invdens,              \
                                          s.counters + 3);                                     \
        break;
    switch (flags & 7) {
        MG_DENS_CASE(1) MG_DENS_CASE(2) MG_DENS_CASE(3) MG_DENS_CASE(4) MG_DENS_CASE(5)
        MG_DENS_CASE(6) MG_DENS_CASE(7)
        default: break;
    }
#undef MG_DENS_CASE
}

// ---- force -------------------------------------------------------------------------------
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

__global__ void __launch_bounds__(256) k_force(DevParams P, Carried C,
                                               const uint32_t* __restrict__ scell,
                                               const uint32_t* __restrict__ count,
                                               const uint32_t* __restrict__ offset,
                                               const float* __restrict__ press,
                                               const float* __restrict__ invdens,
                                               float4* __restrict__ force,
                                               uint32_t* __restrict__ brk,
                                               const uint32_t* __restrict__ nactive_p) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nact = *nactive_p;
    if (p >= nact) return;
    const uint32_t cap = P.cap;
    const float4 ip = C.pos[p], iv = C.veval[p];
    float fx = 0.f, fy = 0.f, fz = 0.f;
    uint32_t br = 0;
    // own (outgoing) bonds
#pragma unroll
    for (int a = 0; a < NB; a++) {
        uint4* rec = C.bond + ((size_t)a * cap + p) * 2;
        const uint4 A = rec[0];
        const uint32_t j = A.x;
        const float restlen = __uint_as_float(A.y);
        if (j >= nact || (double)restlen < 0.000000001) continue;
        const uint4 B = rec[1];
        const float elastlim = __uint_as_float(B.x);
        const BondTerm t = bond_term(ip, iv, C.pos[j], C.veval[j], restlen, __uint_as_float(A.z),
                                     __uint_as_float(A.w), elastlim, P.pmass);
        const float sq = __uint_as_float(B.z) + t.strain * t.strain;
        const float si = __uint_as_float(B.w) + t.strain;
        *reinterpret_cast<uint2*>(&rec[1].z) = make_uint2(__float_as_uint(sq), __float_as_uint(si));
        if (!is_nan3(t)) {
            fx = fx - t.ex;
            fy = fy - t.ey;
            fz = fz - t.ez;
        }
        if (t.absd >= elastlim && !P.freeze) br |= 1u << a;
    }
    // fluid pressure, surface and viscosity terms (contributeForce, cuda:3167-3226)
    {
        const uint32_t base = scell[p] - (uint32_t)P.nadj;
        const float ipress = press[p], idens = invdens[p], sr = P.sr;
        float sx = 0.f, sy = 0.f, sz = 0.f;
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
                if (dsq < 1.f && dsq > 0.f) {
                    const float r = sqrtf(dsq);
                    const float t = sr - r;
                    const float kern = t * t * t;
                    const float prs = 100.f * (ipress + press[q]);
                    const float s = (idens * invdens[q]) * 100.f;
                    const float term = prs * kern - P.surf * (t * t);
                    const float4 jv = C.veval[q];
                    const float px = (s * (dx / r)) * term, py = (s * (dy / r)) * term,
                                pz = (s * (dz / r)) * term;
                    const float vx = (100000.f * (jv.x - iv.x)) * kern;
                    const float vy = (100000.f * (jv.y - iv.y)) * kern;
                    const float vz = (100000.f * (jv.z - iv.z)) * kern;
                    cx = cx + (px + vx);
                    cy = cy + (py + vy);
                    cz = cz + (pz + vz);
                }
            }
            sx = sx + cx;
            sy = sy + cy;
            sz = sz + cz;
        }
        fx = fx + sx * P.pmass;
        fy = fy + sy * P.pmass;
        fz = fz + sz * P.pmass;
    }
    // reactions of incoming bonds, slot order (gather form of the atomicAdd at cuda:3311-3313)
    {
        const uint4* pi = reinterpret_cast<const uint4*>(C.pidx + (size_t)p * 12);
        uint32_t in[12];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            uint4 v = pi[k];
            in[4 * k] = v.x; in[4 * k + 1] = v.y; in[4 * k + 2] = v.z; in[4 * k + 3] = v.w;
        }
#pragma unroll
        for (int b = 0; b < NB; b++) {
            const uint32_t k = in[2 * b], bk = in[2 * b + 1];
            if (k >= nact || bk >= (uint32_t)NB) continue;
            const uint4* rec = C.bond + ((size_t)bk * cap + k) * 2;
            const uint4 A = rec[0];
            if (A.x != p) continue;
            const float restlen = __uint_as_float(A.y);
            if ((double)restlen < 0.000000001) continue;
            const float elastlim = __uint_as_float(reinterpret_cast<const uint32_t*>(rec + 1)[0]);
            const BondTerm t = bond_term(C.pos[k], C.veval[k], ip, iv, restlen,
                                         __uint_as_float(A.z), __uint_as_float(A.w), elastlim,
                                         P.pmass);
            if (!is_nan3(t)) {
                fx = fx + t.ex;
                fy = fy + t.ey;
                fz = fz + t.ez;
            }
        }
    }
    force[p] = make_float4(fx, fy, fz, 0.f);
    brk[p] = br;
}

void launch_force(const DevParams& P, const Carried& cur, const Scratch& s, cudaStream_t st) {
    uint32_t blocks = (P.cap + 255) / 256;
    k_force<<<blocks, 256, 0, st>>>(P, cur, s.scell, s.count, s.offset, s.press, s.invdens,
                                    s.force, s.brk, s.counters + 3);
}

// Broken bonds get rest length 0 (cuda:3315-3317).  The force kernel records the breaks in
// brk[] instead of writing the rest length, because other threads of the same kernel read
// that rest length for their incoming-bond reactions.
__device__ __forceinline__ void apply_breaks(uint4* bond, uint32_t cap, uint32_t p, uint32_t br) {
#pragma unroll
    for (int a = 0; a < NB; a++)
        if (br & (1u << a)) reinterpret_cast<uint32_t*>(bond + ((size_t)a * cap + p) * 2)[1] = 0u;
}

__global__ void __launch_bounds__(256) k_apply_breaks(uint32_t cap, uint4* __restrict__ bond,
                                                      const uint32_t* __restrict__ brk,
                                                      const uint32_t* __restrict__ nactive_p) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p) return;
    const uint32_t br = brk[p];
    if (br) apply_breaks(bond, cap, p, br);
}

void launch_apply_breaks(const DevParams& P, const Carried& cur, const Scratch& s, cudaStream_t st) {
    uint32_t blocks = (P.cap + 255) / 256;
    k_apply_breaks<<<blocks, 256, 0, st>>>(P.cap, cur.bond, s.brk, s.counters + 3);
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

template <bool APPLY_BRK>
__global__ void __launch_bounds__(256) k_advance(DevParams P, Carried C,
                                                 const float4* __restrict__ force,
                                                 const uint32_t* __restrict__ brk,
                                                 const uint32_t* __restrict__ nactive_p) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *nactive_p) return;
    const float4 pos = C.pos[p], ve = C.veval[p], f = force[p];
    float ax = f.x, ay = f.y, az = f.z;
    float diff;
    diff = P.pr - (pos.y - (P.bmin[1] + (pos.x - P.bmin[0]) * P.slope));
    wall(ax, ay, az, diff, -P.slope, P.one_minus_slope, 0.f, P.estiff, P.damp, ve);
    diff = P.pr - (P.bmax[1] - pos.y);
    wall(ax, ay, az, diff, 0.f, -1.f, 0.f, P.estiff, P.damp, ve);
    diff = P.pr - (pos.x - P.bmin[0]);
    wall(ax, ay, az, diff, 1.f, 0.f, 0.f, P.xmin_stiff, P.damp, ve);
    diff = P.pr - (P.bmax[0] - pos.x);
    wall(ax, ay, az, diff, -1.f, 0.f, 0.f, P.xmax_stiff, P.damp, ve);
    diff = P.pr - (pos.z - P.bmin[2]);
    wall(ax, ay, az, diff, 0.f, 0.f, 1.f, P.estiff, P.damp, ve);
    diff = P.pr - (P.bmax[2] - pos.z);
    wall(ax, ay, az, diff, 0.f, 0.f, -1.f, P.estiff, P.damp, ve);
    {
        const float dx = P.bmax[0] - pos.x, dy = P.bmax[1] - pos.y, dz = P.bmax[2] - pos.z;
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
    C.veval[p] = make_float4((vel.x + vnx) * 0.5f, (vel.y + vny) * 0.5f, (vel.z + vnz) * 0.5f, ve.w);
    C.vel[p] = make_float4(vnx, vny, vnz, vel.w);
    C.pos[p] = make_float4(pos.x + vnx * dt, pos.y + vny * dt, pos.z + vnz * dt, pos.w);
    if (APPLY_BRK) {
        const uint32_t br = brk[p];
        if (br) apply_breaks(C.bond, P.cap, p, br);
    }
}

void launch_advance(const DevParams& P, const Carried& cur, const Scratch& s, bool apply_brk,
                    cudaStream_t st) {
    uint32_t blocks = (P.cap + 255) / 256;
    if (apply_brk)
        k_advance<true><<<blocks, 256, 0, st>>>(P, cur, s.force, s.brk, s.counters + 3);
    else
        k_advance<false><<<blocks, 256, 0, st>>>(P, cur, s.force, s.brk, s.counters + 3);
}

}  // namespace mg
