/*
 * ref_harness.cpp - the reference's own per-step kernels compiled as host C++, to pin the
 * oracle (TEST INFRASTRUCTURE ONLY; built into oracle/_ref/ and loaded by the tests).
 *
 * oracle/Makefile copies, from Morphogenesis/src/fluid_system_cuda.cu where it lies, the line
 * ranges of the kernels this harness runs into oracle/_ref/kernels.inc (git-ignored; nothing
 * of the reference is kept in this repository):
 *   insertParticles                      fluid_system_cuda.cu:53-100
 *   countingSortFull                     :196-296
 *   contributePressure, computePressure  :620-712
 *   contributeDiffusion, computeDiffusion :3026-3105
 *   contributeForce, computeForce        :3167-3358
 *   advanceParticles                     :3470-3614
 * and compiles them against the reference's own fluid_system_cuda.cuh, fluid.h and
 * cutil_math.h, with oracle/ref_shim/ standing in for the OpenCL and CUDA headers.
 *
 * Execution: each kernel's body runs once per particle index, one index at a time
 * (ref_host.h).  That is the serial schedule the oracle's canonical decisions name: the
 * atomicAdd arrival rank of insertParticles becomes D1's stable rank, and the float atomicAdd
 * accumulation of computeForce becomes a sum in thread order (D2 gathers instead, so forces
 * agree within rounding, not bitwise).  computeDiffusion updates FCONC in place while other
 * threads read it; the harness gives every thread the pre-pass concentrations (D9, the
 * schedule in which all reads precede all writes).  The reference's genome holds integers
 * (uint diffusability and breakdown rate, fluid.h FGenome), so the pinned scenes use integer
 * rates, on which the oracle's float genome (D3) computes the same values.
 *
 * What is not the reference's code: this sequencing (buffer copies and clears of
 * CountingSortFullCL, host_CUDA.cpp:521-558; TransferPosVelVeval after advanceParticles,
 * host_CL.cpp:199-226), the exclusive scan of the cell counts (prefixSum needs a thread block
 * and shared memory, cuda:136-183; this is a serial scan), and the parameter set-up, which
 * follows FluidParamCL (fluid_system.cpp:521-610) and FluidSetupCL (host_CL.cpp:39-106).
 */
#include "ref_host.h"

// fluid.h's host-side FBufs has no member accessors, but countingSortFull and
// advanceParticles call them (ftemp.bufI(...)); the harness supplies its own FBufs below.
#define FBufs mg_ref_unused_FBufs
#include "fluid_system_cuda.cuh"
#undef FBufs
// cutil_math.h defines its own fminf/fmaxf/min/max unless __OPENCLC__ is set; the CUDA build
// uses CUDA's fmaxf, the IEEE maximum that libm's fmaxf also computes.
#define __OPENCLC__
#include "cutil_math.h"

#include <vector>

#include "mg_oracle.h"

struct FBufs {
    char* mcpu[MAX_BUF];
    uint* bufI(int n) const { return (uint*)mcpu[n]; }
    float* bufF(int n) const { return (float*)mcpu[n]; }
    cl_float3* bufF3(int n) const { return (cl_float3*)mcpu[n]; }
};
static inline uint* bufI(const FBufs* b, int n) { return b->bufI(n); }
static inline float* bufF(const FBufs* b, int n) { return b->bufF(n); }
static inline cl_float3* bufF3(const FBufs* b, int n) { return b->bufF3(n); }

// "no partner" of the reference host and kernels (fluid_system.cpp:22, host_CL.cpp:14; the
// kernel file's own definition is commented out, fluid_system_cuda.cu:49)
#define UINT_MAXSIZE 65535

static FParams fparam;
static FBufs fbuf;
static FBufs ftemp;
static FGenome fgenome;

#include "kernels.inc"

namespace {

struct Store {
    uint32_t n = 0, cells = 0;
    std::vector<uint32_t> a[MAX_BUF];  // fbuf
    std::vector<uint32_t> t[MAX_BUF];  // ftemp
};
Store S;

// 32-bit words of a buffer id (the reference layouts of include/mg_abi.h)
size_t words(int id) {
    const size_t n = S.n, c = S.cells;
    switch (id) {
        case FPOS: case FVEL: case FVEVAL: case FFORCE: return 4 * n;
        case FPRESS: case FDENSITY: case FAGE: case FCOLOR: case FGCELL: case FGNDX: case FBIN:
        case FPARTICLE_ID: case FMASS_RADIUS: case FNERVEIDX: return n;
        case FELASTIDX: return (size_t)BOND_DATA * n;
        case FPARTICLEIDX: return (size_t)BONDS_PER_PARTICLE * 2 * n;
        case FCONC: return (size_t)NUM_TF * n;
        case FEPIGEN: return (size_t)NUM_GENES * n;
        case FBIN_COUNT: case FBIN_OFFSET: return c;
        case FBIN_COUNT_ACTIVE_GENES: return (size_t)NUM_GENES * c;
        default: return 0;
    }
}

const int kParticleBufs[] = {FPOS, FVEL, FVEVAL, FFORCE, FPRESS, FDENSITY, FAGE, FCOLOR, FGCELL,
                             FGNDX, FBIN, FPARTICLE_ID, FMASS_RADIUS, FNERVEIDX, FELASTIDX,
                             FPARTICLEIDX, FCONC, FEPIGEN};

void bind() {
    for (int id = 0; id < MAX_BUF; id++) {
        fbuf.mcpu[id] = S.a[id].empty() ? nullptr : (char*)S.a[id].data();
        ftemp.mcpu[id] = S.t[id].empty() ? nullptr : (char*)S.t[id].data();
    }
}

template <class Body>
void launch(uint32_t n, Body body) {
    blockDim.x = 256;
    blockDim.y = blockDim.z = 1;
    for (uint32_t i = 0; i < n; i++) {
        blockIdx.x = i / 256;
        threadIdx.x = i % 256;
        body();
    }
}

void fill(int id, uint32_t v) {
    for (auto& w : S.a[id]) w = v;
}

}  // namespace

extern "C" {

int mgr_create(const mg_fparams* p, const mg_genome* g, uint32_t n) {
    S = Store();
    S.n = n;
    S.cells = (uint32_t)p->grid_total;
    for (int id = 0; id < MAX_BUF; id++) {
        const size_t w = words(id);
        if (w) {
            S.a[id].assign(w, 0u);
            S.t[id].assign(w, 0u);
        }
    }
    bind();
    memset(&fparam, 0, sizeof(fparam));
    const float ss = p->psimscale, sr = p->psmoothradius, al = p->paccel_limit, vl = p->pvel_limit;
    // FluidParamCL (fluid_system.cpp:521-610)
    fparam.psimscale = ss;
    fparam.psmoothradius = sr;
    fparam.pradius = p->pradius;
    fparam.r2 = sr * sr;
    fparam.pmass = p->pmass;
    fparam.prest_dens = p->prest_dens;
    fparam.pboundmin = make_cl_float3(p->pboundmin[0], p->pboundmin[1], p->pboundmin[2]);
    fparam.pboundmax = make_cl_float3(p->pboundmax[0], p->pboundmax[1], p->pboundmax[2]);
    fparam.pextstiff = p->pextstiff;
    fparam.pintstiff = p->pintstiff;
    fparam.pvisc = p->pvisc;
    fparam.psurface_t = p->psurface_t;
    fparam.pdamp = p->pdamp;
    fparam.pforce_min = p->pforce_min;
    fparam.pforce_max = p->pforce_max;
    fparam.pforce_freq = p->pforce_freq;
    fparam.pground_slope = p->pground_slope;
    fparam.pgravity = make_cl_float3(p->pgravity[0], p->pgravity[1], p->pgravity[2]);
    fparam.AL = al;
    fparam.AL2 = al * al;
    fparam.VL = vl;
    fparam.VL2 = vl * vl;
    fparam.pdist = powf(fparam.pmass / fparam.prest_dens, 1 / 3.0f);
    fparam.wendlandC2kern = 21 / (2 * 3.141592f);
    fparam.H = fparam.psmoothradius / fparam.psimscale;
    fparam.d2 = fparam.psimscale * fparam.psimscale;
    fparam.rd2 = fparam.r2 / fparam.d2;
    fparam.actuation_factor = p->actuation_factor;
    fparam.actuation_period = p->actuation_period;
    // FluidSetupCL (host_CL.cpp:39-106)
    fparam.pnum = (int)n;
    fparam.maxPoints = (int)n;
    fparam.freeze = false;
    fparam.gridRes = make_cl_int3(p->grid_res[0], p->grid_res[1], p->grid_res[2]);
    fparam.gridSize = make_cl_float3(p->grid_size[0], p->grid_size[1], p->grid_size[2]);
    fparam.gridDelta = make_cl_float3(p->grid_delta[0], p->grid_delta[1], p->grid_delta[2]);
    fparam.gridMin = make_cl_float3(p->grid_min[0], p->grid_min[1], p->grid_min[2]);
    fparam.gridMax = make_cl_float3(p->grid_max[0], p->grid_max[1], p->grid_max[2]);
    fparam.gridTotal = p->grid_total;
    const int gs = p->grid_srch;
    fparam.gridSrch = gs;
    fparam.gridAdjCnt = gs * gs * gs;
    fparam.gridScanMax = make_cl_int3(p->grid_res[0] - gs, p->grid_res[1] - gs, p->grid_res[2] - gs);
    int cell = 0;
    for (int y = 0; y < gs; y++)
        for (int z = 0; z < gs; z++)
            for (int x = 0; x < gs; x++)
                fparam.gridAdj[cell++] = (y * fparam.gridRes.z + z) * fparam.gridRes.x + x;
    fparam.debug = 0;
    // the reference genome's integer fields (fluid.h FGenome)
    memset(&fgenome, 0, sizeof(fgenome));
    for (int k = 0; k < NUM_GENES; k++) {
        fgenome.mutability[k] = g->mutability[k];
        fgenome.delay[k] = g->delay[k];
        for (int t = 0; t < NUM_TF; t++) fgenome.sensitivity[k][t] = (uint)g->sensitivity[k][t];
        for (int t = 0; t < 2 * NUM_TF + 1; t++) fgenome.secrete[k][t] = (int)g->secrete[k][t];
        for (int t = 0; t < 2 * NUM_GENES + 1; t++) fgenome.activate[k][t] = (int)g->activate[k][t];
    }
    for (int t = 0; t < NUM_TF; t++) {
        fgenome.tf_diffusability[t] = (uint)g->tf_diffusability[t];
        fgenome.tf_breakdown_rate[t] = (uint)g->tf_breakdown_rate[t];
    }
    memcpy(fgenome.tanh_param, g->tanh_param, sizeof(fgenome.tanh_param));
    memcpy(fgenome.param, g->param, sizeof(fgenome.param));
    return 0;
}

int mgr_import(int32_t id, const void* data, size_t bytes) {
    if (id < 0 || id >= MAX_BUF || words(id) * 4 != bytes) return 1;
    memcpy(S.a[id].data(), data, bytes);
    return 0;
}

int mgr_export(int32_t id, void* data, size_t bytes) {
    if (id < 0 || id >= MAX_BUF || words(id) * 4 != bytes) return 1;
    memcpy(data, S.a[id].data(), bytes);
    return 0;
}

// InsertParticlesCL: cell counts cleared, then insertParticles over every particle.
void mgr_insert(void) {
    fill(FBIN_COUNT, 0u);
    fill(FBIN_COUNT_ACTIVE_GENES, 0u);
    const int n = (int)S.n;
    launch(S.n, [&] { insertParticles(n); });
}

// Exclusive scan of the cell counts (a serial scan in place of prefixSum's block scan).
void mgr_scan(void) {
    uint32_t run = 0;
    for (uint32_t c = 0; c < S.cells; c++) {
        S.a[FBIN_OFFSET][c] = run;
        run += S.a[FBIN_COUNT][c];
    }
}

// CountingSortFullCL (host_CUDA.cpp:521-558): particle buffers to the temporary set, the
// sorted set's bond tables, ids, forces, concentrations and gene words cleared, then
// countingSortFull over every particle.
void mgr_sort(void) {
    for (int id : kParticleBufs) S.t[id] = S.a[id];
    fill(FELASTIDX, UINT_MAXSIZE);
    fill(FPARTICLEIDX, UINT_MAXSIZE);
    fill(FPARTICLE_ID, UINT_MAXSIZE);
    fill(FFORCE, 0u);
    fill(FCONC, 0u);
    fill(FEPIGEN, 0u);
    const int n = (int)S.n;
    launch(S.n, [&] { countingSortFull(n); });
}

void mgr_pressure(void) {
    const int n = (int)S.n;
    launch(S.n, [&] { computePressure(n); });
}

void mgr_force(int freeze) {
    const int n = (int)S.n;
    launch(S.n, [&] { computeForce(n, freeze != 0, 20u); });
}

// computeDiffusion with every thread reading the pre-pass concentrations.
void mgr_diffusion(void) {
    const std::vector<uint32_t> before = S.a[FCONC];
    std::vector<uint32_t> after = before;
    const int n = (int)S.n;
    blockDim.x = 256;
    for (uint32_t i = 0; i < S.n; i++) {
        blockIdx.x = i / 256;
        threadIdx.x = i % 256;
        computeDiffusion(n);
        for (int t = 0; t < NUM_TF; t++) {
            after[(size_t)i * NUM_TF + t] = S.a[FCONC][(size_t)i * NUM_TF + t];
            S.a[FCONC][(size_t)i * NUM_TF + t] = before[(size_t)i * NUM_TF + t];
        }
    }
    S.a[FCONC] = after;
}

// advanceParticles writes the new position, velocity and evaluated velocity to the temporary
// set, which TransferPosVelVeval copies back.
void mgr_advance(float time, float dt, float ss) {
    for (int id : {FPOS, FVEL, FVEVAL}) S.t[id] = S.a[id];
    const int n = (int)S.n;
    launch(S.n, [&] { advanceParticles(time, dt, ss, n); });
    for (int id : {FPOS, FVEL, FVEVAL}) S.a[id] = S.t[id];
}

}  // extern "C"
