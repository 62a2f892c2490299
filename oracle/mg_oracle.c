/*
 * mg_oracle.c - CPU oracle (TEST INFRASTRUCTURE ONLY) of the Morphogenesis step.
 *
 * Restates, in the reference's own expression order, the kernels of
 * Morphogenesis src/fluid_system_cuda.cu and the host sequencing of src/host_CUDA.cpp /
 * src/fluid_system.cpp.  Build flags: -O2 -ffp-contract=off (no fused multiply-add, so a
 * float build evaluates exactly the float operations the reference kernels write).
 *
 * Canonical decisions where the reference is non-deterministic or self-inconsistent
 * (the GPU pipeline implements the same ones):
 *  D1 stable rank: FGNDX[i] = number of earlier-index particles in the same cell
 *     (serial execution of insertParticles, fluid_system_cuda.cu:81).
 *  D2 gather form of the bond reaction: particle j receives +eterm of every bond (k,b) in its
 *     incoming table FPARTICLEIDX whose partner is j, in slot order, after its own force
 *     (replaces atomicAdd, fluid_system_cuda.cu:3311-3313, 3354-3356).
 *  D3 gene kernel: FCONC read as float at [p*16+tf] (fixes cuda:739); secretion accumulated
 *     in float (fixes cuda:747); genome rates/weights float; the tally of ftemp into fbuf is
 *     applied once per living (gene 2) particle (host_CUDA.cpp:696-708 launches it 16 times);
 *     the countdown hand-off to gene+1 is skipped for the last gene (cuda:733 writes past
 *     the buffer).
 *  D4 FELASTIDX word 6 is the float strain-squared integrator (as computeForce uses it).
 *  D6 one step = legacy Run() order (fluid_system.cpp:1179-1349) with one sort per step.
 *  D7 "no partner" is 0xFFFFFFFF (the reference's 65535 collides with valid indices).
 *  D8 particles outside the grid window are dropped by the sort; slots [nactive, N) hold a
 *     parked null particle (advanceParticles' out-of-grid parking, cuda:3474-3477).
 *  D9 diffusion reads the pre-kernel concentrations of all neighbours (Jacobi); the
 *     reference updates FCONC in place while neighbours read it (cuda:3097-3099).
 *  D10 pow(t,3)/pow(t,2) of contributeForce are evaluated as t*t*t and t*t.
 *  D11 pnumActive is the number of particles in the grid window (the reference reads
 *     FBIN_OFFSET at the scan-max corner cell, host_CUDA.cpp:501-511, dropping that cell).
 */
#include "mg_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef MGO_REAL
#define MGO_REAL float
#endif
typedef MGO_REAL real;
#ifdef MGO_DOUBLE
#define RSQRT(x) sqrt(x)
#else
#define RSQRT(x) sqrtf(x)
#endif

#define NB MG_BONDS_PER_PARTICLE
#define NTF MG_NUM_TF
#define NG MG_NUM_GENES
#define EPS_WALL ((real)0.00001f) /* EPSILON, fluid_system_cuda.cuh:41 */

typedef struct { real x, y, z, w; } r4;

typedef struct {
    uint32_t partner; /* [0] current index  */
    real elastlim;    /* [1] elastic limit  */
    real restlen;     /* [2] rest length    */
    real modulus;     /* [3] modulus        */
    real damping;     /* [4] damping coeff  */
    uint32_t pid;     /* [5] particle ID    */
    real sqint;       /* [6] strain^2 integrator (D4) */
    real sint;        /* [7] strain integrator */
    uint32_t change;  /* [8] change type    */
} bond_t;

typedef struct {
    /* FluidParamCL inputs */
    real ss, sr, pr, mass, rest, estiff, istiff, visc, surf, damp, fmin, fmax, ffreq, slope;
    real bmin[3], bmax[3], grav[3], al, vl, a_f, a_p;
    /* FluidSetupCL inputs */
    int32_t res[3], srch, total;
    real gmin[3], gdelta[3];
    /* derived */
    real r2, H, d2, rd2, wc2, AL2, VL2, pdist;
    int32_t scanmax[3], adjcnt, adj[64], nadj;
    real dt, time;
    int32_t freeze;
} params_t;

struct mgo_system {
    uint32_t cap;
    params_t P;
    mg_fparams raw;
    mg_genome G;
    r4 *pos, *vel, *veval, *force;
    real *press, *dens;
    uint32_t *age, *color, *gcell, *gndx, *pid, *mass_radius, *nerve;
    bond_t* bond;     /* [cap][6] */
    uint32_t* pidx;   /* [cap][12] */
    real* conc;       /* [cap][16] */
    uint32_t* epigen; /* [16][cap] */
    uint32_t *count, *offset;           /* [total] */
    uint32_t *gcount, *goffset;         /* [16][total] */
    uint32_t *lists, lens[NG];          /* [16][cap] */
    uint32_t nactive, active_points;
    /* scratch */
    uint32_t* newidx;
    real* conc_new;
    r4* eterm;          /* [cap][6] outgoing eterm, w = 1 if it was applied */
    unsigned char* brk; /* [cap] bonds that broke this step */
    /* changes_valid: computeBondChanges ran since the last sort, so heal takes its slots from
     * the change words (change list 0); heal_params 0 = D5 bond parameters, 1 = makeBond's
     * genome defaults */
    int changes_valid, heal_params;
};

static int g_threads = 0;

int mgo_precision_bits(void) { return (int)(sizeof(real) * 8); }

int mgo_set_threads(int n) {
#ifdef _OPENMP
    g_threads = n > 0 ? n : omp_get_max_threads();
    return g_threads;
#else
    (void)n;
    g_threads = 1;
    return 1;
#endif
}

static int nthreads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

static float bits_to_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f_to_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* ---- a1: derived parameters ------------------------------------------------------------ */
static void derive(params_t* P, const mg_fparams* p) {
    P->ss = p->psimscale; P->sr = p->psmoothradius; P->pr = p->pradius; P->mass = p->pmass;
    P->rest = p->prest_dens; P->estiff = p->pextstiff; P->istiff = p->pintstiff;
    P->visc = p->pvisc; P->surf = p->psurface_t; P->damp = p->pdamp; P->fmin = p->pforce_min;
    P->fmax = p->pforce_max; P->ffreq = p->pforce_freq; P->slope = p->pground_slope;
    for (int k = 0; k < 3; k++) {
        P->bmin[k] = p->pboundmin[k]; P->bmax[k] = p->pboundmax[k]; P->grav[k] = p->pgravity[k];
        P->res[k] = p->grid_res[k]; P->gmin[k] = p->grid_min[k]; P->gdelta[k] = p->grid_delta[k];
    }
    P->al = p->paccel_limit; P->vl = p->pvel_limit; P->a_f = p->actuation_factor;
    P->a_p = p->actuation_period; P->srch = p->grid_srch; P->total = p->grid_total;
    P->dt = p->dt; P->time = p->time; P->freeze = p->freeze;
    /* FluidParamCL, fluid_system.cpp:527-598 */
    P->r2 = P->sr * P->sr;
    P->AL2 = P->al * P->al;
    P->VL2 = P->vl * P->vl;
    P->pdist = (real)pow((double)(P->mass / P->rest), 1.0 / 3.0);
    P->wc2 = (real)21 / ((real)2 * (real)3.141592f);
    P->H = P->sr / P->ss;
    P->d2 = P->ss * P->ss;
    P->rd2 = P->r2 / P->d2;
    /* FluidSetupCL, host_CL.cpp:51-60, 101-106 (same as host_CUDA.cpp:39-54) */
    for (int k = 0; k < 3; k++) P->scanmax[k] = P->res[k] - P->srch;
    int c = 0;
    for (int y = 0; y < P->srch; y++)
        for (int z = 0; z < P->srch; z++)
            for (int x = 0; x < P->srch; x++)
                if (c < 64) P->adj[c++] = (y * P->res[2] + z) * P->res[0] + x;
    P->adjcnt = P->srch * P->srch * P->srch;
    /* computePressure: nadj = (1*res.z + 1)*res.x + 1 (cuda:663) */
    P->nadj = (1 * P->res[2] + 1) * P->res[0] + 1;
}

void mgo_get_derived(mgo_handle h, mgo_derived* o) {
    const params_t* P = &h->P;
    o->r2 = (float)P->r2; o->H = (float)P->H; o->d2 = (float)P->d2; o->rd2 = (float)P->rd2;
    o->wendlandC2kern = (float)P->wc2; o->AL2 = (float)P->AL2; o->VL2 = (float)P->VL2;
    o->pdist = (float)P->pdist;
    for (int k = 0; k < 3; k++) o->gridScanMax[k] = P->scanmax[k];
    o->gridAdjCnt = P->adjcnt;
    for (int k = 0; k < 64; k++) o->gridAdj[k] = k < P->adjcnt ? P->adj[k] : 0;
    o->nadj = P->nadj;
}

float mgo_get_time(mgo_handle h) { return (float)h->P.time; }

/* ---- lifetime -------------------------------------------------------------------------- */
static size_t at_least_one(size_t n) { return n > 0 ? n : 1; }
#define XALLOC(ptr, n) do { (ptr) = calloc(at_least_one((size_t)(n)), sizeof(*(ptr))); if (!(ptr)) goto fail; } while (0)

static void null_particle(mgo_handle h, uint32_t p) {
    const params_t* P = &h->P;
    /* D8: parked like advanceParticles' GRID_UNDEF branch (cuda:3474-3477) */
    h->pos[p].x = P->bmin[0]; h->pos[p].y = P->bmin[1];
    h->pos[p].z = P->bmin[2] - (real)(2 * P->res[2]); h->pos[p].w = 0;
    memset(&h->vel[p], 0, sizeof(r4)); memset(&h->veval[p], 0, sizeof(r4));
    memset(&h->force[p], 0, sizeof(r4));
    h->press[p] = 0; h->dens[p] = 0;
    h->age[p] = 0; h->color[p] = 0; h->gcell[p] = MG_GRID_UNDEF; h->gndx[p] = MG_GRID_UNDEF;
    h->pid[p] = MG_NO_PARTNER; h->mass_radius[p] = 0; h->nerve[p] = 0;
    for (int a = 0; a < NB; a++) {
        bond_t* b = &h->bond[(size_t)p * NB + a];
        memset(b, 0, sizeof(*b));
        b->partner = MG_NO_PARTNER; b->pid = MG_NO_PARTNER;
    }
    for (int k = 0; k < 2 * NB; k++) h->pidx[(size_t)p * 2 * NB + k] = MG_NO_PARTNER;
    for (int t = 0; t < NTF; t++) h->conc[(size_t)p * NTF + t] = 0;
    for (int g = 0; g < NG; g++) h->epigen[(size_t)g * h->cap + p] = 0;
}

mgo_handle mgo_create(const mg_fparams* p, const mg_genome* g, uint32_t cap) {
    if (!p || !g || cap == 0 || p->grid_total <= 0) return NULL;
    if (p->grid_srch < 1 || p->grid_srch > 4) return NULL;
    mgo_handle h = calloc(1, sizeof(*h));
    if (!h) return NULL;
    h->cap = cap;
    h->raw = *p;
    h->G = *g;
    derive(&h->P, p);
    size_t C = (size_t)p->grid_total;
    XALLOC(h->pos, cap); XALLOC(h->vel, cap); XALLOC(h->veval, cap); XALLOC(h->force, cap);
    XALLOC(h->press, cap); XALLOC(h->dens, cap); XALLOC(h->age, cap); XALLOC(h->color, cap);
    XALLOC(h->gcell, cap); XALLOC(h->gndx, cap); XALLOC(h->pid, cap);
    XALLOC(h->mass_radius, cap); XALLOC(h->nerve, cap);
    XALLOC(h->bond, (size_t)cap * NB); XALLOC(h->pidx, (size_t)cap * 2 * NB);
    XALLOC(h->conc, (size_t)cap * NTF); XALLOC(h->epigen, (size_t)cap * NG);
    XALLOC(h->count, C); XALLOC(h->offset, C);
    XALLOC(h->gcount, C * NG); XALLOC(h->goffset, C * NG);
    XALLOC(h->lists, (size_t)cap * NG);
    XALLOC(h->newidx, cap); XALLOC(h->conc_new, (size_t)cap * NTF);
    XALLOC(h->eterm, (size_t)cap * NB); XALLOC(h->brk, cap);
    for (uint32_t i = 0; i < cap; i++) {
        h->gcell[i] = MG_GRID_UNDEF; h->gndx[i] = MG_GRID_UNDEF;
        for (int a = 0; a < NB; a++) { h->bond[(size_t)i * NB + a].partner = MG_NO_PARTNER; h->bond[(size_t)i * NB + a].pid = MG_NO_PARTNER; }
        for (int k = 0; k < 2 * NB; k++) h->pidx[(size_t)i * 2 * NB + k] = MG_NO_PARTNER;
    }
    memset(h->lists, 0xFF, sizeof(uint32_t) * (size_t)cap * NG);
    h->nactive = cap;
    return h;
fail:
    mgo_destroy(h);
    return NULL;
}

void mgo_destroy(mgo_handle h) {
    if (!h) return;
    free(h->pos); free(h->vel); free(h->veval); free(h->force); free(h->press); free(h->dens);
    free(h->age); free(h->color); free(h->gcell); free(h->gndx); free(h->pid);
    free(h->mass_radius); free(h->nerve); free(h->bond); free(h->pidx); free(h->conc);
    free(h->epigen); free(h->count); free(h->offset); free(h->gcount); free(h->goffset);
    free(h->lists); free(h->newidx); free(h->conc_new); free(h->eterm); free(h->brk);
    free(h);
}

int mgo_update_params(mgo_handle h, const mg_fparams* p) {
    if (p->grid_total != h->raw.grid_total) return 1;
    h->raw = *p;
    derive(&h->P, p);
    return 0;
}

int mgo_update_genome(mgo_handle h, const mg_genome* g) { h->G = *g; return 0; }

void mgo_get_counts(mgo_handle h, uint32_t* n, uint32_t* a) {
    if (n) *n = h->nactive;
    if (a) *a = h->active_points;
}

/* ---- buffer exchange --------------------------------------------------------------------- */
static int copy_r4_in(r4* dst, const void* src, uint32_t n) {
    const float* s = (const float*)src;
    for (uint32_t i = 0; i < n; i++) {
        dst[i].x = s[4 * i]; dst[i].y = s[4 * i + 1]; dst[i].z = s[4 * i + 2]; dst[i].w = s[4 * i + 3];
    }
    return 0;
}
static void copy_r4_out(void* dst, const r4* src, uint32_t n) {
    float* d = (float*)dst;
    for (uint32_t i = 0; i < n; i++) {
        d[4 * i] = (float)src[i].x; d[4 * i + 1] = (float)src[i].y;
        d[4 * i + 2] = (float)src[i].z; d[4 * i + 3] = (float)src[i].w;
    }
}

int mgo_import(mgo_handle h, int32_t id, const void* data, size_t bytes) {
    uint32_t n = h->cap;
    size_t C = (size_t)h->P.total;
    switch (id) {
    case MG_FPOS: if (bytes != 16ull * n) return 1; return copy_r4_in(h->pos, data, n);
    case MG_FVEL: if (bytes != 16ull * n) return 1; return copy_r4_in(h->vel, data, n);
    case MG_FVEVAL: if (bytes != 16ull * n) return 1; return copy_r4_in(h->veval, data, n);
    case MG_FFORCE: if (bytes != 16ull * n) return 1; return copy_r4_in(h->force, data, n);
    case MG_FPRESS: case MG_FDENSITY: {
        if (bytes != 4ull * n) return 1;
        real* d = id == MG_FPRESS ? h->press : h->dens;
        const float* s = (const float*)data;
        for (uint32_t i = 0; i < n; i++) d[i] = s[i];
        return 0;
    }
    case MG_FAGE: case MG_FCOLOR: case MG_FPARTICLE_ID: case MG_FMASS_RADIUS: case MG_FNERVEIDX: {
        if (bytes != 4ull * n) return 1;
        uint32_t* d = id == MG_FAGE ? h->age : id == MG_FCOLOR ? h->color : id == MG_FPARTICLE_ID ? h->pid
                    : id == MG_FMASS_RADIUS ? h->mass_radius : h->nerve;
        memcpy(d, data, bytes);
        return 0;
    }
    case MG_FELASTIDX: {
        if (bytes != 4ull * n * MG_BOND_DATA) return 1;
        const uint32_t* s = (const uint32_t*)data;
        for (size_t k = 0; k < (size_t)n * NB; k++) {
            const uint32_t* w = s + k * MG_DATA_PER_BOND;
            bond_t* b = &h->bond[k];
            b->partner = w[0]; b->elastlim = bits_to_f(w[1]); b->restlen = bits_to_f(w[2]);
            b->modulus = bits_to_f(w[3]); b->damping = bits_to_f(w[4]); b->pid = w[5];
            b->sqint = bits_to_f(w[6]); b->sint = bits_to_f(w[7]); b->change = w[8];
        }
        return 0;
    }
    case MG_FPARTICLEIDX: if (bytes != 4ull * n * 2 * NB) return 1; memcpy(h->pidx, data, bytes); return 0;
    case MG_FCONC: {
        if (bytes != 4ull * n * NTF) return 1;
        const float* s = (const float*)data;
        for (size_t k = 0; k < (size_t)n * NTF; k++) h->conc[k] = s[k];
        return 0;
    }
    case MG_FEPIGEN: if (bytes != 4ull * n * NG) return 1; memcpy(h->epigen, data, bytes); return 0;
    case MG_FGCELL: if (bytes != 4ull * n) return 1; memcpy(h->gcell, data, bytes); return 0;
    case MG_FGNDX: if (bytes != 4ull * n) return 1; memcpy(h->gndx, data, bytes); return 0;
    case MG_FBIN_COUNT: if (bytes != 4 * C) return 1; memcpy(h->count, data, bytes); return 0;
    case MG_FBIN_OFFSET: if (bytes != 4 * C) return 1; memcpy(h->offset, data, bytes); return 0;
    default: return 2;
    }
}

/* Change lists (countingSortChanges, cuda:406-618) from the bonds' change words: bin by bin,
 * the bin's particles in sorted order, each particle's bonds in slot order, one entry
 * (particle, bond) in list k for bit k of the change word.  counts / offsets are [9][cells],
 * lists [9][2][cap] (particle row, then bond row; unused entries 0xFFFFFFFF), lengths [9]. */
static void change_lists(mgo_handle h, uint32_t* counts, uint32_t* offsets, uint32_t* lists,
                         uint32_t* lengths) {
    const size_t C = (size_t)h->P.total, cap = h->cap;
    const uint32_t n = h->nactive;
    if (counts) memset(counts, 0, 4 * C * MG_NUM_CHANGES);
    if (offsets) memset(offsets, 0, 4 * C * MG_NUM_CHANGES);
    if (lists) memset(lists, 0xFF, 8 * cap * MG_NUM_CHANGES);
    uint32_t len[MG_NUM_CHANGES] = {0};
    for (size_t c = 0; c < C; c++) {
        for (int k = 0; k < MG_NUM_CHANGES; k++)
            if (offsets) offsets[k * C + c] = len[k];
        const uint32_t last = h->offset[c] + h->count[c];
        for (uint32_t p = h->offset[c]; p < last && p < n; p++)
            for (int b = 0; b < NB; b++) {
                const uint32_t w = h->bond[(size_t)p * NB + b].change;
                for (int k = 0; k < MG_NUM_CHANGES; k++)
                    if ((w >> k) & 1u) {
                        if (counts) counts[k * C + c]++;
                        if (lists) {
                            lists[(size_t)k * 2 * cap + len[k]] = p;
                            lists[(size_t)k * 2 * cap + cap + len[k]] = (uint32_t)b;
                        }
                        len[k]++;
                    }
            }
    }
    if (lengths) memcpy(lengths, len, sizeof len);
}

int mgo_export(mgo_handle h, int32_t id, void* data, size_t bytes) {
    uint32_t n = h->cap;
    size_t C = (size_t)h->P.total;
    switch (id) {
    case MG_FPOS: if (bytes != 16ull * n) return 1; copy_r4_out(data, h->pos, n); return 0;
    case MG_FVEL: if (bytes != 16ull * n) return 1; copy_r4_out(data, h->vel, n); return 0;
    case MG_FVEVAL: if (bytes != 16ull * n) return 1; copy_r4_out(data, h->veval, n); return 0;
    case MG_FFORCE: if (bytes != 16ull * n) return 1; copy_r4_out(data, h->force, n); return 0;
    case MG_FPRESS: case MG_FDENSITY: {
        if (bytes != 4ull * n) return 1;
        const real* s = id == MG_FPRESS ? h->press : h->dens;
        float* d = (float*)data;
        for (uint32_t i = 0; i < n; i++) d[i] = (float)s[i];
        return 0;
    }
    case MG_FAGE: case MG_FCOLOR: case MG_FPARTICLE_ID: case MG_FMASS_RADIUS: case MG_FNERVEIDX:
    case MG_FGCELL: case MG_FGNDX: {
        if (bytes != 4ull * n) return 1;
        const uint32_t* s = id == MG_FAGE ? h->age : id == MG_FCOLOR ? h->color : id == MG_FPARTICLE_ID ? h->pid
                          : id == MG_FMASS_RADIUS ? h->mass_radius : id == MG_FNERVEIDX ? h->nerve
                          : id == MG_FGCELL ? h->gcell : h->gndx;
        memcpy(data, s, bytes);
        return 0;
    }
    case MG_FBIN: {
        if (bytes != 4ull * n) return 1;
        uint32_t* d = (uint32_t*)data; /* countingSortFull: FBIN[sort_ndx] = sort_ndx (cuda:225) */
        for (uint32_t i = 0; i < n; i++) d[i] = i < h->nactive ? i : MG_GRID_UNDEF;
        return 0;
    }
    case MG_FELASTIDX: {
        if (bytes != 4ull * n * MG_BOND_DATA) return 1;
        uint32_t* d = (uint32_t*)data;
        for (size_t k = 0; k < (size_t)n * NB; k++) {
            uint32_t* w = d + k * MG_DATA_PER_BOND;
            const bond_t* b = &h->bond[k];
            w[0] = b->partner; w[1] = f_to_bits((float)b->elastlim); w[2] = f_to_bits((float)b->restlen);
            w[3] = f_to_bits((float)b->modulus); w[4] = f_to_bits((float)b->damping); w[5] = b->pid;
            w[6] = f_to_bits((float)b->sqint); w[7] = f_to_bits((float)b->sint); w[8] = b->change;
        }
        return 0;
    }
    case MG_FPARTICLEIDX: if (bytes != 4ull * n * 2 * NB) return 1; memcpy(data, h->pidx, bytes); return 0;
    case MG_FCONC: {
        if (bytes != 4ull * n * NTF) return 1;
        float* d = (float*)data;
        for (size_t k = 0; k < (size_t)n * NTF; k++) d[k] = (float)h->conc[k];
        return 0;
    }
    case MG_FEPIGEN: if (bytes != 4ull * n * NG) return 1; memcpy(data, h->epigen, bytes); return 0;
    case MG_FBIN_COUNT: if (bytes != 4 * C) return 1; memcpy(data, h->count, bytes); return 0;
    case MG_FBIN_OFFSET: if (bytes != 4 * C) return 1; memcpy(data, h->offset, bytes); return 0;
    case MG_FBIN_COUNT_ACTIVE_GENES: if (bytes != 4 * C * NG) return 1; memcpy(data, h->gcount, bytes); return 0;
    case MG_FBIN_OFFSET_ACTIVE_GENES: if (bytes != 4 * C * NG) return 1; memcpy(data, h->goffset, bytes); return 0;
    case MG_FDENSE_LIST_LENGTHS: if (bytes != 4 * NG) return 1; memcpy(data, h->lens, bytes); return 0;
    case MG_FDENSE_LISTS: if (bytes != 4ull * n * NG) return 1; memcpy(data, h->lists, bytes); return 0;
    case MG_FBIN_COUNT_CHANGES: if (bytes != 4 * C * MG_NUM_CHANGES) return 1; change_lists(h, (uint32_t*)data, NULL, NULL, NULL); return 0;
    case MG_FBIN_OFFSET_CHANGES: if (bytes != 4 * C * MG_NUM_CHANGES) return 1; change_lists(h, NULL, (uint32_t*)data, NULL, NULL); return 0;
    case MG_FDENSE_LIST_LENGTHS_CHANGES: if (bytes != 4 * MG_NUM_CHANGES) return 1; change_lists(h, NULL, NULL, NULL, (uint32_t*)data); return 0;
    case MG_FDENSE_LISTS_CHANGES: if (bytes != 8ull * n * MG_NUM_CHANGES) return 1; change_lists(h, NULL, NULL, (uint32_t*)data, NULL); return 0;
    default: return 2;
    }
}

int mgo_export_f64(mgo_handle h, int32_t id, double* out, size_t count) {
    uint32_t n = h->cap;
    const r4* v = NULL;
    switch (id) {
    case MG_FPOS: v = h->pos; break;
    case MG_FVEL: v = h->vel; break;
    case MG_FVEVAL: v = h->veval; break;
    case MG_FFORCE: v = h->force; break;
    case MG_FPRESS: case MG_FDENSITY: {
        if (count != n) return 1;
        const real* s = id == MG_FPRESS ? h->press : h->dens;
        for (uint32_t i = 0; i < n; i++) out[i] = (double)s[i];
        return 0;
    }
    case MG_FCONC:
        if (count != (size_t)n * NTF) return 1;
        for (size_t k = 0; k < count; k++) out[k] = (double)h->conc[k];
        return 0;
    case MG_FELASTIDX:
        if (count != (size_t)n * MG_BOND_DATA) return 1;
        for (size_t k = 0; k < (size_t)n * NB; k++) {
            double* w = out + k * MG_DATA_PER_BOND;
            const bond_t* b = &h->bond[k];
            w[0] = 0; w[1] = b->elastlim; w[2] = b->restlen; w[3] = b->modulus; w[4] = b->damping;
            w[5] = 0; w[6] = b->sqint; w[7] = b->sint; w[8] = 0;
        }
        return 0;
    default: return 2;
    }
    if (count != 4ull * n) return 1;
    for (uint32_t i = 0; i < n; i++) {
        out[4 * i] = v[i].x; out[4 * i + 1] = v[i].y; out[4 * i + 2] = v[i].z; out[4 * i + 3] = v[i].w;
    }
    return 0;
}

/* ---- a2: insertParticles (fluid_system_cuda.cu:53-100) ---------------------------------- */
/* Cell of a position: gcf = (pos - gridMin) * gridDelta, truncated; valid when
 * 1 <= gc <= gridScanMax per axis (cuda:70-79).  Written as float comparisons so NaN and
 * huge values fall outside the window without an undefined float->int conversion. */
static uint32_t cell_of(const params_t* P, const r4* p) {
    real gx = (p->x - P->gmin[0]) * P->gdelta[0];
    real gy = (p->y - P->gmin[1]) * P->gdelta[1];
    real gz = (p->z - P->gmin[2]) * P->gdelta[2];
    if (!(gx >= (real)1 && gx < (real)(P->scanmax[0] + 1))) return MG_GRID_UNDEF;
    if (!(gy >= (real)1 && gy < (real)(P->scanmax[1] + 1))) return MG_GRID_UNDEF;
    if (!(gz >= (real)1 && gz < (real)(P->scanmax[2] + 1))) return MG_GRID_UNDEF;
    int cx = (int)gx, cy = (int)gy, cz = (int)gz;
    return (uint32_t)((cy * P->res[2] + cz) * P->res[0] + cx);
}

void mgo_insert_particles(mgo_handle h) {
    const params_t* P = &h->P;
    size_t C = (size_t)P->total;
    memset(h->count, 0, 4 * C);  /* InsertParticlesCL zeroes the counts first */
    memset(h->gcount, 0, 4 * C * NG);
    for (uint32_t i = 0; i < h->cap; i++) {
        uint32_t gs = cell_of(P, &h->pos[i]);
        h->gcell[i] = gs;
        if (gs == MG_GRID_UNDEF) { h->gndx[i] = MG_GRID_UNDEF; continue; }
        h->gndx[i] = h->count[gs]++; /* D1: serial order = stable rank */
        for (int g = 0; g < NG; g++)
            if (h->epigen[(size_t)g * h->cap + i] > 0) h->gcount[(size_t)g * C + gs]++;
    }
}

/* ---- a3: prefixSum/prefixFixup (cuda:136-183), zero_offsets=1 => exclusive -------------- */
static uint32_t exclusive_scan(const uint32_t* in, uint32_t* out, size_t n) {
    uint32_t run = 0;
    for (size_t k = 0; k < n; k++) { out[k] = run; run += in[k]; }
    return run;
}

void mgo_prefix_sum_cells(mgo_handle h) {
    const params_t* P = &h->P;
    size_t C = (size_t)P->total;
    h->nactive = exclusive_scan(h->count, h->offset, C);
    for (int g = 0; g < NG; g++) exclusive_scan(h->gcount + g * C, h->goffset + g * C, C);
    /* mActivePoints = FBIN_OFFSET[grid_ScanMax] (host_CUDA.cpp:501-505), reported only */
    int corner = (P->scanmax[1] * P->res[2] + P->scanmax[2]) * P->res[0] + P->scanmax[0];
    h->active_points = (corner >= 0 && (size_t)corner < C) ? h->offset[corner] : h->nactive;
}

/* ---- a4/a5: countingSortFull (cuda:196-296) + countingSortDenseLists (cuda:329-404) -------- */
#define PERMUTE(field, type, per)                                                   \
    do {                                                                            \
        type* nf = malloc(sizeof(type) * (size_t)cap * (per));                      \
        if (!nf) return;                                                            \
        for (uint32_t i = 0; i < cap; i++) {                                        \
            uint32_t s = h->newidx[i];                                              \
            if (s == MG_GRID_UNDEF) continue;                                       \
            memcpy(nf + (size_t)s * (per), h->field + (size_t)i * (per), sizeof(type) * (per)); \
        }                                                                           \
        free(h->field); h->field = nf;                                              \
    } while (0)

void mgo_counting_sort_full(mgo_handle h) {
    const params_t* P = &h->P;
    h->changes_valid = 0;
    uint32_t cap = h->cap;
    size_t C = (size_t)P->total;
    /* sort_ndx = FBIN_OFFSET[icell] + FGNDX (cuda:210-211) */
    for (uint32_t i = 0; i < cap; i++) {
        uint32_t c = h->gcell[i];
        h->newidx[i] = c == MG_GRID_UNDEF ? MG_GRID_UNDEF : h->offset[c] + h->gndx[i];
    }
    /* bond partner remap through the old->new permutation (cuda:230-244) */
    for (uint32_t i = 0; i < cap; i++) {
        if (h->newidx[i] == MG_GRID_UNDEF) continue;
        for (int a = 0; a < NB; a++) {
            bond_t* b = &h->bond[(size_t)i * NB + a];
            uint32_t j = b->partner, js = MG_NO_PARTNER;
            if (j < cap && h->newidx[j] != MG_GRID_UNDEF && h->newidx[j] < cap) js = h->newidx[j];
            b->partner = js;
        }
        /* incoming list remap (cuda:256-268) */
        for (int a = 0; a < NB; a++) {
            uint32_t* w = &h->pidx[(size_t)i * 2 * NB + 2 * a];
            uint32_t k = w[0], ks = MG_NO_PARTNER;
            if (k < cap && h->newidx[k] != MG_GRID_UNDEF) ks = h->newidx[k];
            w[0] = ks;
        }
    }
    uint32_t* sorted_cell = malloc(4ull * cap);
    uint32_t* sorted_ndx = malloc(4ull * cap);
    if (!sorted_cell || !sorted_ndx) { free(sorted_cell); free(sorted_ndx); return; }
    for (uint32_t i = 0; i < cap; i++) {
        uint32_t s = h->newidx[i];
        if (s == MG_GRID_UNDEF) continue;
        sorted_cell[s] = h->gcell[i];
        sorted_ndx[s] = h->gndx[i];
    }
    PERMUTE(pos, r4, 1); PERMUTE(vel, r4, 1); PERMUTE(veval, r4, 1);
    PERMUTE(press, real, 1); PERMUTE(dens, real, 1); PERMUTE(age, uint32_t, 1);
    PERMUTE(color, uint32_t, 1); PERMUTE(pid, uint32_t, 1); PERMUTE(mass_radius, uint32_t, 1);
    PERMUTE(nerve, uint32_t, 1); PERMUTE(bond, bond_t, NB); PERMUTE(pidx, uint32_t, 2 * NB);
    PERMUTE(conc, real, NTF);
    {   /* FEPIGEN is [gene][particle] */
        uint32_t* ne = malloc(4ull * cap * NG);
        if (!ne) { free(sorted_cell); free(sorted_ndx); return; }
        for (uint32_t i = 0; i < cap; i++) {
            uint32_t s = h->newidx[i];
            if (s == MG_GRID_UNDEF) continue;
            for (int g = 0; g < NG; g++) ne[(size_t)g * cap + s] = h->epigen[(size_t)g * cap + i];
        }
        free(h->epigen); h->epigen = ne;
    }
    for (uint32_t s = 0; s < h->nactive; s++) {
        h->gcell[s] = sorted_cell[s];
        h->gndx[s] = sorted_ndx[s];
        memset(&h->force[s], 0, sizeof(r4)); /* FFORCE = 0 (cuda:219) */
    }
    free(sorted_cell); free(sorted_ndx);
    for (uint32_t s = h->nactive; s < cap; s++) null_particle(h, s);
    /* dense lists: per gene, sorted indices of particles with FEPIGEN>0, bin by bin */
    memset(h->lists, 0xFF, 4ull * cap * NG);
    for (int g = 0; g < NG; g++) {
        uint32_t len = 0;
        for (uint32_t s = 0; s < h->nactive; s++)
            if (h->epigen[(size_t)g * cap + s] > 0) h->lists[(size_t)g * cap + len++] = s;
        /* tally_denselist_lengths: len = cnt[last] + off[last] (cuda:185-194) */
        h->lens[g] = h->gcount[(size_t)g * C + C - 1] + h->goffset[(size_t)g * C + C - 1];
        (void)len;
    }
}

/* ---- a6: contributePressure / computePressure (cuda:620-712) ------------------------------- */
void mgo_compute_pressure(mgo_handle h) {
    const params_t* P = &h->P;
    const int n = (int)h->nactive;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int i = 0; i < n; i++) {
        uint32_t gc = h->gcell[i];
        if (gc == MG_GRID_UNDEF) continue;
        gc -= (uint32_t)P->nadj;
        r4 p = h->pos[i];
        real sum = 0;
        for (int c = 0; c < P->adjcnt; c++) {
            uint32_t cell = gc + (uint32_t)P->adj[c];
            if (h->count[cell] == 0) continue;
            real part = 0;
            uint32_t clast = h->offset[cell] + h->count[cell];
            for (uint32_t j = h->offset[cell]; j < clast; j++) {
                real dx = p.x - h->pos[j].x, dy = p.y - h->pos[j].y, dz = p.z - h->pos[j].z;
                real dsq = dx * dx + dy * dy + dz * dz;
                if (dsq < P->r2 && dsq > (real)0) {
                    real r = RSQRT(dsq);
                    real q = r / P->sr;
                    real b = (real)1 - q;
                    b *= b;
                    b *= b;
                    part += b * ((real)4 * q + (real)1);
                }
            }
            sum += part;
        }
        sum = sum * P->mass * P->wc2;
        if (sum == (real)0) sum = (real)1;
        h->press[i] = (sum - P->rest) * P->istiff;
        h->dens[i] = (real)1 / sum;
    }
}

/* ---- a7: contributeForce / computeForce (cuda:3167-3358) ---------------------------------- */
/* eterm of bond slot a of particle i (cuda:3263-3307); returns 1 when the reference would
 * apply it (partner in range, rest length > 1e-9, no NaN component). */
static int bond_eterm(mgo_handle h, uint32_t i, int a, uint32_t nact, r4* et, real* strain_out,
                      real* absd_out) {
    const params_t* P = &h->P;
    const bond_t* b = &h->bond[(size_t)i * NB + a];
    uint32_t j = b->partner;
    if (j >= nact || (double)b->restlen < 0.000000001) return -1; /* float vs double literal (cuda:3268) */
    real dx = h->pos[i].x - h->pos[j].x, dy = h->pos[i].y - h->pos[j].y, dz = h->pos[i].z - h->pos[j].z;
    real dsq = dx * dx + dy * dy + dz * dz;
    real absd = RSQRT(dsq) + (real)FLT_MIN;
    real rvx = h->veval[j].x - h->veval[i].x, rvy = h->veval[j].y - h->veval[i].y,
         rvz = h->veval[j].z - h->veval[i].z;
    real q = (absd - b->restlen) / b->restlen;
    real strain = q > (real)0 ? q : (real)0; /* fmaxf(0, q): NaN -> 0 */
    real flag = (real)(absd < b->elastlim);
    et->x = (flag * (((dx / absd) * strain) * b->modulus - b->damping * rvx)) / P->mass;
    et->y = (flag * (((dy / absd) * strain) * b->modulus - b->damping * rvy)) / P->mass;
    et->z = (flag * (((dz / absd) * strain) * b->modulus - b->damping * rvz)) / P->mass;
    et->w = 0;
    *strain_out = strain;
    *absd_out = absd;
    return (et->x != et->x || et->y != et->y || et->z != et->z) ? 0 : 1;
}

void mgo_compute_force(mgo_handle h) {
    const params_t* P = &h->P;
    const int n = (int)h->nactive;
    const uint32_t nact = h->nactive;
    /* phase 1: own bonds, integrators, breaks, fluid force */
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int ii = 0; ii < n; ii++) {
        uint32_t i = (uint32_t)ii;
        h->brk[i] = 0;
        if (h->gcell[i] == MG_GRID_UNDEF) continue;
        r4 force = {0, 0, 0, 0};
        for (int a = 0; a < NB; a++) {
            r4* et = &h->eterm[(size_t)i * NB + a];
            real strain = 0, absd = 0;
            int ok = bond_eterm(h, i, a, nact, et, &strain, &absd);
            et->w = 0;
            if (ok < 0) continue;
            bond_t* b = &h->bond[(size_t)i * NB + a];
            b->sqint = b->sqint + strain * strain;
            b->sint = b->sint + strain;
            if (ok == 1) {
                force.x = force.x - et->x; force.y = force.y - et->y; force.z = force.z - et->z;
                et->w = 1;
            }
            if (absd >= b->elastlim && !P->freeze) h->brk[i] |= (unsigned char)(1u << a);
        }
        /* fluid (cuda:3339-3346, contributeForce 3167-3226) */
        uint32_t gc = h->gcell[i] - (uint32_t)P->nadj;
        r4 ip = h->pos[i], iv = h->veval[i];
        real ipress = h->press[i], idens = h->dens[i], sr = P->sr;
        real fx = 0, fy = 0, fz = 0;
        for (int c = 0; c < P->adjcnt; c++) {
            uint32_t cell = gc + (uint32_t)P->adj[c];
            if (h->count[cell] == 0) continue;
            real cx = 0, cy = 0, cz = 0;
            uint32_t clast = h->offset[cell] + h->count[cell];
            for (uint32_t j = h->offset[cell]; j < clast; j++) {
                real dx = ip.x - h->pos[j].x, dy = ip.y - h->pos[j].y, dz = ip.z - h->pos[j].z;
                real dsq = dx * dx + dy * dy + dz * dz;
                real r = RSQRT(dsq);
                if (dsq < (real)1 && dsq > (real)0) {
                    real t = sr - r;
                    real kern = t * t * t;
                    real press = (real)100 * (ipress + h->press[j]);
                    real s = (idens * h->dens[j]) * (real)100;
                    real term = press * kern - P->surf * (t * t);
                    real px = (s * (dx / r)) * term, py = (s * (dy / r)) * term, pz = (s * (dz / r)) * term;
                    real vx = ((real)100000 * (h->veval[j].x - iv.x)) * kern;
                    real vy = ((real)100000 * (h->veval[j].y - iv.y)) * kern;
                    real vz = ((real)100000 * (h->veval[j].z - iv.z)) * kern;
                    cx = cx + (px + vx); cy = cy + (py + vy); cz = cz + (pz + vz);
                }
            }
            fx = fx + cx; fy = fy + cy; fz = fz + cz;
        }
        force.x = force.x + fx * P->mass;
        force.y = force.y + fy * P->mass;
        force.z = force.z + fz * P->mass;
        h->force[i] = force;
    }
    /* phase 2 (D2): reactions of incoming bonds, slot order */
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int ii = 0; ii < n; ii++) {
        uint32_t i = (uint32_t)ii;
        if (h->gcell[i] == MG_GRID_UNDEF) continue;
        r4 f = h->force[i];
        for (int b = 0; b < NB; b++) {
            uint32_t k = h->pidx[(size_t)i * 2 * NB + 2 * b];
            uint32_t bk = h->pidx[(size_t)i * 2 * NB + 2 * b + 1];
            if (k >= nact || bk >= NB) continue;
            if (h->bond[(size_t)k * NB + bk].partner != i) continue;
            const r4* et = &h->eterm[(size_t)k * NB + bk];
            if (et->w == 0) continue;
            f.x = f.x + et->x; f.y = f.y + et->y; f.z = f.z + et->z;
        }
        h->force[i] = f;
    }
    /* broken bonds: rest length 0 (cuda:3315-3317) */
    for (uint32_t i = 0; i < nact; i++)
        if (h->brk[i])
            for (int a = 0; a < NB; a++)
                if (h->brk[i] & (1u << a)) h->bond[(size_t)i * NB + a].restlen = 0;
}

/* ---- a8: contributeDiffusion / computeDiffusion (cuda:3026-3105), D9 Jacobi --------------- */
void mgo_compute_diffusion(mgo_handle h) {
    const params_t* P = &h->P;
    const int n = (int)h->nactive;
    const mg_genome* G = &h->G;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int ii = 0; ii < n; ii++) {
        uint32_t i = (uint32_t)ii;
        real* out = h->conc_new + (size_t)i * NTF;
        const real* cur = h->conc + (size_t)i * NTF;
        if (h->gcell[i] == MG_GRID_UNDEF) { memcpy(out, cur, sizeof(real) * NTF); continue; }
        real nc[NTF];
        real diff[NTF];
        for (int t = 0; t < NTF; t++) { nc[t] = 0; diff[t] = G->tf_diffusability[t]; }
        real d2 = P->ss * P->ss;
        real r2 = P->r2 / d2;
        uint32_t gc = h->gcell[i] - (uint32_t)P->nadj;
        r4 p = h->pos[i];
        for (int c = 0; c < P->adjcnt; c++) {
            uint32_t cell = gc + (uint32_t)P->adj[c];
            if (h->count[cell] == 0) continue;
            uint32_t clast = h->offset[cell] + h->count[cell];
            for (uint32_t j = h->offset[cell]; j < clast; j++) {
                real dx = p.x - h->pos[j].x, dy = p.y - h->pos[j].y, dz = p.z - h->pos[j].z;
                real dsq = dx * dx + dy * dy + dz * dz;
                if (dsq < r2 && dsq > (real)0) {
                    real cc = (r2 - dsq) * d2;
                    const real* cj = h->conc + (size_t)j * NTF;
                    for (int t = 0; t < NTF; t++)
                        if (diff[t] != (real)0) nc[t] += (diff[t] * cc) * (cj[t] - cur[t]);
                }
            }
        }
        for (int t = 0; t < NTF; t++) out[t] = (real)G->tf_breakdown_rate[t] * (cur[t] + nc[t]);
    }
    for (uint32_t i = 0; i < h->nactive; i++)
        memcpy(h->conc + (size_t)i * NTF, h->conc_new + (size_t)i * NTF, sizeof(real) * NTF);
}

/* ---- a9: computeGeneAction + tallyGeneAction (cuda:714-772), D3 -------------------------- */
void mgo_compute_genes(mgo_handle h) {
    const int n = (int)h->nactive;
    const mg_genome* G = &h->G;
    const uint32_t cap = h->cap;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int ii = 0; ii < n; ii++) {
        uint32_t p = (uint32_t)ii;
        uint32_t E0[NG], E[NG], dE[NG];
        real dconc[NTF];
        real* conc = h->conc + (size_t)p * NTF;
        for (int g = 0; g < NG; g++) { E0[g] = E[g] = h->epigen[(size_t)g * cap + p]; dE[g] = 0; }
        for (int t = 0; t < NTF; t++) dconc[t] = 0;
        for (int g = 0; g < NG; g++) {
            if (E0[g] == 0) continue; /* not in dense list g */
            int delay = (int)E[g];
            if (0 < delay && delay < INT_MAX) {
                E[g]--;
                if (delay == 1 && g + 1 < NG && E[g + 1] != 0) E[g + 1] = G->delay[g + 1];
            }
            real act = 0;
            for (int t = 0; t < NTF; t++)
                if (G->sensitivity[g][t] != 0.0f) act += (real)G->sensitivity[g][t] * conc[t];
            int ns = (int)G->secrete[g][2 * NTF];
            for (int k = 0; k < ns && k < NTF; k++) {
                int tf = (int)G->secrete[g][2 * k];
                if (tf < 0 || tf >= NTF) continue;
                dconc[tf] += (real)G->secrete[g][2 * k + 1] * act;
            }
            int na = (int)G->activate[g][2 * NG];
            for (int k = 0; k < na && k < NG; k++) {
                int og = (int)G->activate[g][2 * k];
                if (og < 0 || og >= NG) continue;
                if ((real)G->activate[g][2 * k + 1] < act) dE[og] += 1;
            }
        }
        if (E0[2] != 0) { /* tally over the living list (dense list 2) */
            for (int t = 0; t < NTF; t++) conc[t] += dconc[t];
            for (int g = 0; g < NG; g++) E[g] += dE[g];
        }
        for (int g = 0; g < NG; g++) h->epigen[(size_t)g * cap + p] = E[g];
    }
}

/* ---- a10: advanceParticles (cuda:3470-3614) ----------------------------------------------- */
static inline void wall(r4* accel, real diff, real nx, real ny, real nz, real stiff, real damp, const r4* ve) {
    if (diff > EPS_WALL) {
        real adj = stiff * diff - damp * (nx * ve->x + ny * ve->y + nz * ve->z);
        accel->x = accel->x + nx * adj; accel->y = accel->y + ny * adj; accel->z = accel->z + nz * adj;
    }
}

void mgo_advance(mgo_handle h) {
    const params_t* P = &h->P;
    const int n = (int)h->nactive;
    const real dt = P->dt;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int ii = 0; ii < n; ii++) {
        uint32_t i = (uint32_t)ii;
        if (h->gcell[i] == MG_GRID_UNDEF) {
            h->pos[i].x = P->bmin[0]; h->pos[i].y = P->bmin[1]; h->pos[i].z = P->bmin[2] - (real)(2 * P->res[2]);
            h->vel[i].x = h->vel[i].y = h->vel[i].z = 0;
            continue;
        }
        r4 pos = h->pos[i], ve = h->veval[i];
        r4 accel = h->force[i];
        real diff;
        diff = P->pr - (pos.y - (P->bmin[1] + (pos.x - P->bmin[0]) * P->slope));
        wall(&accel, diff, -P->slope, (real)1 - P->slope, 0, P->estiff, P->damp, &ve);
        diff = P->pr - (P->bmax[1] - pos.y);
        wall(&accel, diff, 0, -1, 0, P->estiff, P->damp, &ve);
        diff = P->pr - (pos.x - P->bmin[0]);
        wall(&accel, diff, 1, 0, 0, (P->fmin + (real)1) * P->estiff, P->damp, &ve);
        diff = P->pr - (P->bmax[0] - pos.x);
        wall(&accel, diff, -1, 0, 0, (P->fmax + (real)1) * P->estiff, P->damp, &ve);
        diff = P->pr - (pos.z - P->bmin[2]);
        wall(&accel, diff, 0, 0, 1, P->estiff, P->damp, &ve);
        diff = P->pr - (P->bmax[2] - pos.z);
        wall(&accel, diff, 0, 0, -1, P->estiff, P->damp, &ve);
        {   /* shield (cuda:3540-3547) */
            real dx = P->bmax[0] - pos.x, dy = P->bmax[1] - pos.y, dz = P->bmax[2] - pos.z;
            diff = (real)2 * P->pr - (dx + dy + dz);
            wall(&accel, diff, 1, 1, 1, P->estiff, P->damp, &ve);
        }
        accel.x = accel.x + P->grav[0]; accel.y = accel.y + P->grav[1]; accel.z = accel.z + P->grav[2];
        real speed = accel.x * accel.x + accel.y * accel.y + accel.z * accel.z;
        if (speed > P->AL2) {
            real s = P->al / RSQRT(speed);
            accel.x *= s; accel.y *= s; accel.z *= s;
        }
        r4 vel = h->vel[i];
        speed = vel.x * vel.x + vel.y * vel.y + vel.z * vel.z;
        if (speed > P->VL2) { /* speed = VL2; vel *= VL/sqrt(speed) (cuda:3576-3579) */
            real s = P->vl / RSQRT(P->VL2);
            vel.x *= s; vel.y *= s; vel.z *= s;
        }
        r4 vn;
        vn.x = accel.x * dt + vel.x; vn.y = accel.y * dt + vel.y; vn.z = accel.z * dt + vel.z;
        h->veval[i].x = (vel.x + vn.x) * (real)0.5; h->veval[i].y = (vel.y + vn.y) * (real)0.5;
        h->veval[i].z = (vel.z + vn.z) * (real)0.5;
        h->vel[i].x = vn.x; h->vel[i].y = vn.y; h->vel[i].z = vn.z;
        h->pos[i].x = pos.x + vn.x * dt; h->pos[i].y = pos.y + vn.y * dt; h->pos[i].z = pos.z + vn.z * dt;
    }
    h->P.time = h->P.time + dt; /* AdvanceTime (fluid_system.cpp:2016) */
}

/* ---- a11 (D5): re-forming of broken bonds ---------------------------------------------------
 * Deterministic restatement of heal's bond-0 rule (contribFindBonds theta = dsq, cuda:1938-1975;
 * heal cuda:2047-2105 without the curand jitter of cuda:2066-2071; makeBond cuda:1573-1593):
 *  - a slot is broken when its partner is an active particle and its rest length failed the
 *    computeForce rest-length test (cuda:3268; breaks set the rest length to 0, cuda:3316);
 *  - each particle with a broken slot proposes, for its lowest broken slot, the nearest particle
 *    j within h (dsq < rd2, dsq > 0) that is not a boundary marker (particle id 0, cuda:1950),
 *    is not already the partner of any of its slots (cuda:1960) and has a free incoming slot
 *    (fewer than six live incoming bonds); ties go to the lower sorted index;
 *  - every particle accepts proposals in (distance, index) order into its free incoming slots,
 *    in slot order; the others retry on a later step;
 *  - the new bond: rest length = current distance, elastic limit 1.5 x rest length (strain
 *    0.5), modulus and damping kept from the broken slot, integrators and change word 0,
 *    word 5 = the partner's particle id (makeBond's [5]). */
static int rest_is_small(real r) { return (double)r < 0.000000001; }

/* The slot a particle heals this call, or -1.  Without bond changes (D5): its lowest slot
 * whose partner is active and whose rest length failed the rest-length test.  After
 * computeBondChanges: its lowest slot in change list 0 (change word bit 0, the order
 * countingSortChanges lists them, cuda:470-490) that still needs a bond (rest length 0 or no
 * active partner: a bond made since is not replaced). */
static int heal_slot(const mgo_handle h, uint32_t i, uint32_t n) {
    for (int a = 0; a < NB; a++) {
        const bond_t* b = &h->bond[(size_t)i * NB + a];
        if (h->changes_valid) {
            if ((b->change & 1u) && (b->restlen == (real)0 || b->partner >= n)) return a;
        } else if (b->partner < n && rest_is_small(b->restlen)) {
            return a;
        }
    }
    return -1;
}

/* Deterministic tanh for computeBondChanges, the same float operations as the GPU kernel:
 * |x| < 0.5: odd Taylor polynomial through x^15 (Horner in x^2); 0.5 <= |x| < 9:
 * 1 - 2 / (exp(2|x|) + 1) with exp by Cody-Waite reduction (ln 2 split in a 16-bit head and a
 * tail) and a degree-8 Taylor polynomial scaled by 2^k; beyond 9, +-1.  Error <= 2 ulp. */
static float fbits(uint32_t u) { union { uint32_t u; float f; } v = {u}; return v.f; }
float mgo_tanh_cw(float x) {
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

#ifdef MGO_DOUBLE
#define RTANH(x) tanh(x)
#else
#define RTANH(x) mgo_tanh_cw(x)
#endif

/* ---- a11: computeBondChanges (cuda:1065-1331) over the living list (dense list 2) ----------
 * Bond types from the tissue genes (cuda:1127-1132; the cartilage branch tests gene 6 again
 * and is never taken); per bond in slot order: a bond with rest length > 0 averages its strain
 * integrators over the inner-loop steps, zeroes them, and scales rest length and modulus by
 * the genome's shifted tanh (l_a + l_b tanh(l_c s - l_d), s_a + s_b tanh(s_c s2 - s_d),
 * cuda:1156-1207); its change word is zeroed; the first bond with rest length 0 or no partner
 * (any index outside the active particles) is flagged for heal (change word 1) and ends the
 * particle's loop (cuda:1214-1244).  Lengthen/shorten/strengthen/weaken flags are never set by
 * the reference (their insertion is commented out, cuda:1245-1285), so lists 1-8 stay empty. */
void mgo_compute_bond_changes(mgo_handle h, uint32_t steps) {
    const uint32_t n = h->nactive, cap = h->cap;
    const mg_genome* G = &h->G;
    const real fsteps = (real)(float)steps;
    const uint32_t len = h->lens[2];
    for (uint32_t li = 0; li < len; li++) {
        const uint32_t i = h->lists[(size_t)2 * cap + li];
        if (i >= n) continue;
        int type[NB] = {0, 0, 0, 0, 0, 0};
        const uint32_t* E = h->epigen;
        if (E[(size_t)9 * cap + i] > 0) { type[0] = type[1] = type[2] = type[3] = 2; }
        else if (E[(size_t)6 * cap + i] > 0 || E[(size_t)7 * cap + i] > 0 || E[(size_t)10 * cap + i] > 0) type[0] = 1;
        for (int b = 0; b < NB; b++) {
            bond_t* B = &h->bond[(size_t)i * NB + b];
            if (B->restlen > (real)0) {
                const real si = B->sint / fsteps, sq = B->sqint / fsteps;
                B->sint = 0;
                B->sqint = 0;
                const float* T = G->tanh_param[type[b]];
                B->restlen *= (real)T[0] + (real)T[1] * RTANH((real)T[2] * si - (real)T[3]);
                B->modulus *= (real)T[4] + (real)T[5] * RTANH((real)T[6] * sq - (real)T[7]);
            }
            B->change = 0;
            if (B->restlen == (real)0 || B->partner >= n) {
                B->change += 1;
                break;
            }
        }
    }
    h->changes_valid = 1;
}

void mgo_set_heal_params(mgo_handle h, int mode) { h->heal_params = mode; }

void mgo_remodel(mgo_handle h) {
    const params_t* P = &h->P;
    const uint32_t n = h->nactive;
    if (n == 0) return;
    unsigned char* freemask = (unsigned char*)calloc(n, 1);
    uint32_t* prop = (uint32_t*)malloc(sizeof(uint32_t) * n);
    real* propd = (real*)malloc(sizeof(real) * n);
    for (uint32_t j = 0; j < n; j++) {
        unsigned m = 0;
        for (int s = 0; s < NB; s++) {
            uint32_t k = h->pidx[(size_t)j * 2 * NB + 2 * s], bk = h->pidx[(size_t)j * 2 * NB + 2 * s + 1];
            int live = k < n && bk < NB && h->bond[(size_t)k * NB + bk].partner == j &&
                       !rest_is_small(h->bond[(size_t)k * NB + bk].restlen);
            if (!live) m |= 1u << s;
        }
        freemask[j] = (unsigned char)m;
    }
    for (uint32_t i = 0; i < n; i++) {
        prop[i] = MG_GRID_UNDEF;
        propd[i] = 0;
        if (h->gcell[i] == MG_GRID_UNDEF || heal_slot(h, i, n) < 0) continue;
        const r4 ip = h->pos[i];
        const uint32_t gc = h->gcell[i] - (uint32_t)P->nadj;
        real best = 0;
        uint32_t bj = MG_GRID_UNDEF;
        for (int c = 0; c < P->adjcnt; c++) {
            uint32_t cell = gc + (uint32_t)P->adj[c];
            uint32_t clast = h->offset[cell] + h->count[cell];
            for (uint32_t j = h->offset[cell]; j < clast; j++) {
                real dx = ip.x - h->pos[j].x, dy = ip.y - h->pos[j].y, dz = ip.z - h->pos[j].z;
                real dsq = dx * dx + dy * dy + dz * dz;
                if (!(dsq < P->rd2 && dsq > (real)0)) continue;
                if (h->pid[j] == 0 || freemask[j] == 0) continue;
                int bonded = 0;
                for (int a = 0; a < NB; a++) bonded |= h->bond[(size_t)i * NB + a].partner == j;
                if (bonded) continue;
                if (bj == MG_GRID_UNDEF || dsq < best) { best = dsq; bj = j; }
            }
        }
        prop[i] = bj;
        propd[i] = best;
    }
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t j = prop[i];
        if (j == MG_GRID_UNDEF) continue;
        const real d = propd[i];
        uint32_t rank = 0;
        const uint32_t gc = h->gcell[j] - (uint32_t)P->nadj;
        for (int c = 0; c < P->adjcnt; c++) {
            uint32_t cell = gc + (uint32_t)P->adj[c];
            uint32_t clast = h->offset[cell] + h->count[cell];
            for (uint32_t q = h->offset[cell]; q < clast; q++)
                if (prop[q] == j && (propd[q] < d || (propd[q] == d && q < i))) rank++;
        }
        unsigned m = freemask[j];
        uint32_t r = rank;
        int slot = -1;
        for (int s = 0; s < NB; s++)
            if ((m >> s) & 1u) {
                if (r == 0) { slot = s; break; }
                r--;
            }
        if (slot < 0) continue;
        const int b = heal_slot(h, i, n);
        bond_t* nb = &h->bond[(size_t)i * NB + b];
        nb->partner = j;
        if (h->heal_params) { /* makeBond(i, j, b, slot, elastin) (cuda:1573-1593) */
            const float* E = h->G.param[0];
            nb->elastlim = (real)E[8];
            nb->restlen = (real)E[9];
            nb->modulus = (real)E[10];
            nb->damping = (real)E[11];
        } else {
            const real rest = RSQRT(d);
            nb->restlen = rest;
            nb->elastlim = (real)1.5f * rest;
        }
        nb->pid = h->pid[j];
        nb->sqint = 0;
        nb->sint = 0;
        nb->change = 0;
        h->pidx[(size_t)j * 2 * NB + 2 * slot] = i;
        h->pidx[(size_t)j * 2 * NB + 2 * slot + 1] = (uint32_t)b;
    }
    free(freemask);
    free(prop);
    free(propd);
}

/* ---- SpecialParticlesCL (host_CUDA.cpp:869-900): externalActuation (cuda:3617-3691) for gene
 * 12, then fixedParticles (cuda:3694-3705) for gene 11, applied to the integrated state ------
 * The sine is a Cody-Waite reduction (pi/2 in three float parts, the first two with 12
 * significant bits) with Taylor polynomials of degree 9 / 8, in separate float operations, the
 * same expression the GPU kernel evaluates. */
static float sin_cw(float x) {
    const float P1 = 1.5703125f;
    union { uint32_t u; float f; } p2 = {0x39fda000u}, p3 = {0x33a22169u};
    if (x - x != 0.0f) return x - x; /* NaN or infinity: NaN */
    const float k = rintf(x * 0.636619772f);
    const float r = ((x - k * P1) - k * p2.f) - k * p3.f;
    const int q = (int)k & 3;
    const float s = r * r;
    const float sn = r + r * s * ((-1.0f / 6.0f) + s * ((1.0f / 120.0f) + s * ((-1.0f / 5040.0f) + s * (1.0f / 362880.0f))));
    const float cs = 1.0f + s * (-0.5f + s * ((1.0f / 24.0f) + s * ((-1.0f / 720.0f) + s * (1.0f / 40320.0f))));
    return q == 0 ? sn : q == 1 ? cs : q == 2 ? -sn : -cs;
}

static void special_particles(mgo_handle h, const r4* pos0, const r4* vel0, const r4* veval0,
                              real time) {
    const params_t* P = &h->P;
    for (uint32_t i = 0; i < h->nactive; i++) {
        const int act = h->epigen[(size_t)12 * h->cap + i] != 0, fixed = h->epigen[(size_t)11 * h->cap + i] != 0;
        if (act) {
            const float ph = (float)time / ((float)P->a_p * (float)P->dt);
            h->pos[i] = pos0[i];
            h->pos[i].z = pos0[i].z + P->a_f * (real)sin_cw(ph);
            h->vel[i] = vel0[i];
            h->veval[i] = veval0[i];
        }
        if (fixed) {
            h->pos[i] = pos0[i];
            h->vel[i] = vel0[i];
            h->veval[i] = veval0[i];
        }
    }
}

/* ---- D6: one step in the legacy Run() order --------------------------------------------- */
void mgo_step(mgo_handle h, uint32_t nsteps, uint32_t flags) {
    int saved_freeze = h->P.freeze;
    if (flags & MG_STEP_FREEZE) h->P.freeze = 1;
    for (uint32_t s = 0; s < nsteps; s++) {
        mgo_insert_particles(h);
        mgo_prefix_sum_cells(h);
        mgo_counting_sort_full(h);
        if (flags & MG_STEP_PHYSICS) {
            mgo_compute_pressure(h);
            mgo_compute_force(h);
        }
        if (flags & MG_STEP_GENES) {
            mgo_compute_diffusion(h);
            mgo_compute_genes(h);
        }
        if (flags & MG_STEP_BOND_CHANGES) mgo_compute_bond_changes(h, 1); /* ComputeBondChangesCL */
        if (flags & (MG_STEP_REMODEL | MG_STEP_BOND_CHANGES)) mgo_remodel(h); /* heal, before AdvanceCL */
        if (flags & MG_STEP_PHYSICS) {
            r4 *p0 = NULL, *v0 = NULL, *e0 = NULL;
            const real t = h->P.time;
            if (flags & MG_STEP_SPECIAL) {
                p0 = (r4*)malloc(sizeof(r4) * (h->nactive + 1));
                v0 = (r4*)malloc(sizeof(r4) * (h->nactive + 1));
                e0 = (r4*)malloc(sizeof(r4) * (h->nactive + 1));
                memcpy(p0, h->pos, sizeof(r4) * h->nactive);
                memcpy(v0, h->vel, sizeof(r4) * h->nactive);
                memcpy(e0, h->veval, sizeof(r4) * h->nactive);
            }
            mgo_advance(h);
            if (flags & MG_STEP_SPECIAL) {
                special_particles(h, p0, v0, e0, t);
                free(p0); free(v0); free(e0);
            }
        }
    }
    h->P.freeze = saved_freeze;
}
