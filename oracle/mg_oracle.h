/*
 * mg_oracle.h - CPU oracle of the Morphogenesis per-timestep particle pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference kernels
 * (Morphogenesis src/fluid_system_cuda.cu) and of their host sequencing
 * (src/host_CUDA.cpp, src/fluid_system.cpp), used by tests/, by smoke() and by the
 * CPU-baseline leg of bench.py as the checker.  It is never linked into the product.
 *
 * Parity status: pinned by the reference's own kernels.  The reference ships no tests or golden
 * vectors and its compute path does not build as a program here (fluid_system_cuda.cu needs
 * <CL/cl.h>; the OpenCL host needs jsoncpp/VTK/an ICD), but its insertParticles,
 * countingSortFull, computePressure, computeForce, computeDiffusion and advanceParticles compile
 * as host C++ against stand-ins for the OpenCL/CUDA headers (oracle/ref_harness.cpp, built into
 * oracle/_ref/).  The tests compare this restatement with them stage by stage (bit-exact except
 * the force sums, D2) and keep their outputs as golden vectors (tests/golden/ref_pins.json).
 * The gene reaction (D3) and bond re-forming (D5, D12) differ from the reference by design and
 * are pinned by known-answer tests hand-derived from the reference formulas (tests/golden/).
 *
 * The same source builds twice: MGO_REAL=float (liboracle_f32, expression order of the
 * reference kernels, no FMA contraction) and MGO_REAL=double (liboracle_f64, the "FP64 host
 * oracle" used for error reports).  Both take and return the reference buffer layouts of
 * include/mg_abi.h through mgo_import/mgo_export.
 */
#ifndef MG_ORACLE_H
#define MG_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/mg_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mgo_system* mgo_handle;

/* Derived constants exposed for the a1 parity check (fluid_system.cpp:521-610,
 * host_CL.cpp:39-106).  All values are float regardless of the build. */
typedef struct mgo_derived {
    float r2, H, d2, rd2, wendlandC2kern, AL2, VL2, pdist;
    int32_t gridScanMax[3];
    int32_t gridAdjCnt;
    int32_t gridAdj[64];
    int32_t nadj;
} mgo_derived;

int mgo_precision_bits(void); /* 32 or 64 */
mgo_handle mgo_create(const mg_fparams* p, const mg_genome* g, uint32_t max_points);
void mgo_destroy(mgo_handle h);
int mgo_update_params(mgo_handle h, const mg_fparams* p);
int mgo_update_genome(mgo_handle h, const mg_genome* g);
void mgo_get_derived(mgo_handle h, mgo_derived* out);
float mgo_get_time(mgo_handle h);

/* Buffer exchange in the reference layouts (same ids and bytes as mg_upload/mg_download). */
int mgo_import(mgo_handle h, int32_t buf_id, const void* data, size_t bytes);
int mgo_export(mgo_handle h, int32_t buf_id, void* data, size_t bytes);
/* Float fields at full precision: FPOS/FVEL/FVEVAL/FFORCE (N*4), FPRESS/FDENSITY (N),
 * FCONC (N*16), FELASTIDX float words (N*54, integer words as 0). */
int mgo_export_f64(mgo_handle h, int32_t buf_id, double* out, size_t count);
void mgo_get_counts(mgo_handle h, uint32_t* num_points, uint32_t* active_points);

/* Stages. */
void mgo_insert_particles(mgo_handle h);
void mgo_prefix_sum_cells(mgo_handle h);
void mgo_counting_sort_full(mgo_handle h);
void mgo_compute_pressure(mgo_handle h);
void mgo_compute_force(mgo_handle h);
void mgo_compute_diffusion(mgo_handle h);
void mgo_compute_genes(mgo_handle h);
void mgo_advance(mgo_handle h);
void mgo_remodel(mgo_handle h); /* D5 re-forming of broken bonds (Run2Remodelling) */
/* computeBondChanges over the living list with steps_per_InnerPhysicalLoop = steps; the next
 * mgo_remodel heals the slots it flagged */
void mgo_compute_bond_changes(mgo_handle h, uint32_t steps);
/* bond parameters of healed bonds: 0 = D5 (rest length = distance, elastic limit 1.5 x rest,
 * modulus and damping kept), 1 = makeBond's elastin defaults from the genome */
void mgo_set_heal_params(mgo_handle h, int mode);
float mgo_tanh_cw(float x); /* the deterministic tanh computeBondChanges uses */
/* nsteps steps in the legacy Run() order, flags as mg_step. */
void mgo_step(mgo_handle h, uint32_t nsteps, uint32_t flags);

/* OpenMP threads used by the parallel stages (0 = runtime default); returns the count. */
int mgo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
