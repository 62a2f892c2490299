/*
 * mg_abi.h - C-ABI of the GB300 per-timestep particle pipeline (Morphogenesis drop-in).
 *
 * This is the boundary a host program links against in place of the reference's
 * FluidSystem compute backend (Morphogenesis src/host_CL.cpp, src/host_CUDA.cpp and the
 * FluidSystem run/transfer methods in src/fluid_system.cpp).  Every entry point is plain C:
 * host pointers and sizes in, an mg_status out.  No CUDA or torch types appear here.
 *
 * Ownership: a handle owns all device memory for its particles and grid (the reference's
 * FluidSystem owns mgpu[] per buffer id, fluid.h:239-242).  Host pointers are borrowed for
 * the duration of a call only.  Errors are returned, never exit()ed; mg_last_error() gives
 * the text.  A handle is single-threaded (one CUDA stream, like the reference's one
 * in-order queue, fluid_system.h:365); distinct handles may be used from distinct threads.
 *
 * Buffer ids are numerically equal to the reference's F* ids (fluid.h:138-206) and the bytes
 * exchanged by mg_upload/mg_download use the reference's device element layouts:
 *   FPOS/FVEL/FVEVAL/FFORCE  float[N][4]            (cl_float3, 16 bytes)
 *   FPRESS/FDENSITY          float[N]               (FDENSITY holds 1/density)
 *   FAGE/FCOLOR/FGCELL/FGNDX/FBIN/FPARTICLE_ID/FMASS_RADIUS/FNERVEIDX  uint32[N]
 *   FELASTIDX                uint32[N][6][9]        (words 1-4 and 6-7 are float bits)
 *   FPARTICLEIDX             uint32[N][12]          ((particle, bond) pairs of incoming bonds)
 *   FCONC                    float[N][16]           (device layout used by the kernels; or
 *                                                   float[16][N], getConc's, with MG_OPT_CONC_LAYOUT)
 *   FEPIGEN                  uint32[16][N]          ([gene][particle])
 *   FBIN_COUNT/FBIN_OFFSET   uint32[grid_total]
 *   FBIN_COUNT_ACTIVE_GENES/FBIN_OFFSET_ACTIVE_GENES  uint32[16][grid_total]
 *   FDENSE_LIST_LENGTHS      uint32[16]
 *   FDENSE_LISTS             uint32[16][N]          (list g padded with 0xFFFFFFFF)
 * N is the max_points given to mg_create (the reference's mMaxPoints).
 */
#ifndef MG_ABI_H
#define MG_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- sizes (fluid.h:72-103) ---------------------------------------------------------- */
#define MG_BONDS_PER_PARTICLE 6
#define MG_DATA_PER_BOND 9
#define MG_BOND_DATA (MG_BONDS_PER_PARTICLE * MG_DATA_PER_BOND)
#define MG_NUM_TF 16
#define MG_NUM_GENES 16
#define MG_NUM_CHANGES 9
#define MG_GRID_UNDEF 0xFFFFFFFFu   /* fluid_system_cuda.cuh:43 */
/* "No bond" partner index.  The reference writes UINT_MAXSIZE=65535 (fluid_system.cpp:22),
 * which is a valid particle index once N > 65535; any index >= N means "no bond" on input
 * and the pipeline writes this value. */
#define MG_NO_PARTNER 0xFFFFFFFFu
#define MG_EPIGEN_ACTIVE 2147483647u /* INT_MAX, "fixedActive" (fluid_system.cpp:1110) */

/* ---- buffer ids (fluid.h:138-206) ------------------------------------------------------- */
enum mg_buf {
    MG_FPOS = 0, MG_FVEL = 1, MG_FVEVAL = 2, MG_FFORCE = 3, MG_FPRESS = 4, MG_FDENSITY = 5,
    MG_FAGE = 6, MG_FCOLOR = 7, MG_FGCELL = 8, MG_FGNDX = 9, MG_FGNEXT = 10, MG_FNBRNDX = 11,
    MG_FNBRCNT = 12, MG_FCLUSTER = 13, MG_FELASTIDX = 14, MG_FNERVEIDX = 15, MG_FCONC = 16,
    MG_FEPIGEN = 17, MG_FBIN = 18, MG_FBIN_COUNT = 19, MG_FBIN_OFFSET = 20, MG_FBIN_ACT = 21,
    MG_FSTATE = 22, MG_FPARAMS = 24, MG_FAUXARRAY1 = 25, MG_FAUXSCAN1 = 26, MG_FAUXARRAY2 = 27,
    MG_FAUXSCAN2 = 28, MG_FPARTICLEIDX = 29, MG_FPARTICLE_ID = 30, MG_FMASS_RADIUS = 31,
    MG_FBIN_COUNT_ACTIVE_GENES = 32, MG_FBIN_OFFSET_ACTIVE_GENES = 33,
    MG_FDENSE_LIST_LENGTHS = 34, MG_FDENSE_LISTS = 35, MG_FDENSE_BUF_LENGTHS = 36,
    MG_FBIN_OFFSET_CHANGES = 37, MG_FBIN_COUNT_CHANGES = 38, MG_FDENSE_LIST_LENGTHS_CHANGES = 39,
    MG_FDENSE_LISTS_CHANGES = 40, MG_FDENSE_BUF_LENGTHS_CHANGES = 41, MG_FCURAND_STATE = 42,
    MG_FCURAND_SEED = 43, MG_MAX_BUF = 44
};

/* ---- scalar parameter ids for mg_set_param (fluid_system.h:77-103) --------------------- */
enum mg_param {
    MG_PSIMSCALE = 4, MG_PVISC = 7, MG_PRESTDENSITY = 8, MG_PMASS = 9, MG_PRADIUS = 10,
    MG_PSMOOTHRADIUS = 12, MG_PINTSTIFF = 13, MG_PEXTSTIFF = 14, MG_PEXTDAMP = 15,
    MG_PACCEL_LIMIT = 16, MG_PVEL_LIMIT = 17, MG_PGROUND_SLOPE = 19, MG_PFORCE_MIN = 20,
    MG_PFORCE_MAX = 21, MG_PFORCE_FREQ = 23, MG_PSURFACE_TENSION = 24,
    MG_PACTUATION_FACTOR = 25, MG_PACTUATION_PERIOD = 26,
    /* run controls with no m_Param id in the reference (m_DT, m_Time, FParams.freeze) */
    MG_PDT = 100, MG_PTIME = 101, MG_PFREEZE = 102
};

typedef enum mg_status {
    MG_OK = 0,
    MG_ERR_INVALID_ARG = 1,
    MG_ERR_OOM = 2,
    MG_ERR_GRID_OVERFLOW = 3,   /* a grid cell holds more particles than the sort supports */
    MG_ERR_LIST_OVERFLOW = 4,
    MG_ERR_DEVICE_TIMEOUT = 5,  /* a bounded device-side wait gave up */
    MG_ERR_CUDA = 6,
    MG_ERR_UNSUPPORTED = 7,
    MG_ERR_INCONSISTENT = 8     /* uploaded state violates an invariant the pipeline needs */
} mg_status;

/* Flags for mg_step. */
enum mg_step_flags {
    MG_STEP_PHYSICS = 1u << 0,   /* pressure, force, advance */
    MG_STEP_GENES = 1u << 1,     /* diffusion + gene reaction */
    MG_STEP_REMODEL = 1u << 2,   /* bond break/re-form (heal) */
    MG_STEP_FREEZE = 1u << 3,    /* bonds do not break this step (FParams.freeze) */
    MG_STEP_SURROGATE = 1u << 4, /* learned reaction instead of the plain gene reaction */
    MG_STEP_SPECIAL = 1u << 5,   /* SpecialParticlesCL after the integration: gene 12 particles are
                                    actuated (externalActuation), gene 11 particles stay fixed
                                    (fixedParticles), fluid_system_cuda.cu:3617-3705 */
    MG_STEP_BOND_CHANGES = 1u << 6, /* computeBondChanges (steps_per_InnerPhysicalLoop 1) before
                                       the heal, which then heals the slots it flagged; implies
                                       MG_STEP_REMODEL (legacy Run(), fluid_system.cpp:1256) */
    MG_STEP_DEFAULT = MG_STEP_PHYSICS | MG_STEP_GENES
};

/*
 * Simulation parameters: the arguments of FluidParamCL (fluid_system.cpp:521) and of
 * FluidSetupCL (host_CL.cpp:39), plus the run controls m_DT, m_Time and freeze.
 * Derived constants (r2, H, d2, rd2, AL2, VL2, Wendland normalisation, gridAdj, gridScanMax)
 * are computed inside the library exactly as FluidParamCL/FluidSetupCL compute them.
 */
typedef struct mg_fparams {
    float psimscale;         /* ss */
    float psmoothradius;     /* sr, simulation units */
    float pradius;           /* pr */
    float pmass;
    float prest_dens;
    float pboundmin[3];
    float pboundmax[3];
    float pextstiff;
    float pintstiff;
    float pvisc;
    float psurface_t;
    float pdamp;
    float pforce_min;
    float pforce_max;
    float pforce_freq;
    float pground_slope;
    float pgravity[3];
    float paccel_limit;      /* al */
    float pvel_limit;        /* vl */
    float actuation_factor;  /* a_f */
    float actuation_period;  /* a_p */
    int32_t grid_res[3];
    int32_t grid_srch;       /* gsrch: 1-D neighbour search width (2..4) */
    float grid_size[3];
    float grid_delta[3];
    float grid_min[3];
    float grid_max[3];
    int32_t grid_total;
    float dt;                /* m_DT */
    float time;              /* m_Time */
    int32_t freeze;          /* FParams.freeze */
    int32_t debug;
} mg_fparams;

/*
 * Genome (fluid.h:398-422) with the fields the gene kernel reads as fractions widened to
 * float: sensitivity is a signed weight, diffusability and breakdown are rates, and the
 * secrete/activate sparse lists hold (index, value) pairs with the count in entry [2*16];
 * indices and counts are small exact integers stored as float.
 */
typedef struct mg_genome {
    uint32_t mutability[MG_NUM_GENES];
    uint32_t delay[MG_NUM_GENES];
    float sensitivity[MG_NUM_GENES][MG_NUM_TF];
    float tf_diffusability[MG_NUM_TF];
    float tf_breakdown_rate[MG_NUM_TF];
    float secrete[MG_NUM_GENES][2 * MG_NUM_TF + 1];
    float activate[MG_NUM_GENES][2 * MG_NUM_GENES + 1];
    float tanh_param[3][8];
    float param[3][12];
} mg_genome;

typedef struct mg_system* mg_handle;

/* ---- host-only helpers (no GPU needed) ------------------------------------------------- */

/* SetupGrid (fluid_system.cpp:2073-2131): fills grid_res/size/delta/min/max/total/srch of p
 * from the volume corners, the cell size in simulation units and p->psmoothradius /
 * p->psimscale.  gsrch_override > 0 replaces the computed search width, as FluidSetupCL's
 * own gsrch argument does (host_CL.cpp:39,55). */
mg_status mg_setup_grid(mg_fparams* p, const float vol_min[3], const float vol_max[3],
                        float cell_size, int32_t gsrch_override);

/* Library version string. */
const char* mg_version(void);

/* Last error text of a handle (or of the calling thread when h is NULL). */
const char* mg_last_error(mg_handle h);

/* ---- lifetime (FluidSetupCL + AllocateParticles + AllocateGrid, host_CL.cpp:39-174) ---- */
mg_status mg_create(const mg_fparams* params, const mg_genome* genome, uint32_t max_points,
                    mg_handle* out);
mg_status mg_destroy(mg_handle h);

/* UpdateParams / FluidParamCL (fluid_system.cpp:521-610): grid fields must match creation. */
mg_status mg_update_params(mg_handle h, const mg_fparams* params);
/* UpdateGenome (fluid_system.cpp:494). */
mg_status mg_update_genome(mg_handle h, const mg_genome* genome);
/* SetParam(id, value) on m_Param ids (fluid_system.h:77-103) plus MG_PDT/MG_PTIME/MG_PFREEZE. */
mg_status mg_set_param(mg_handle h, int32_t param_id, float value);
mg_status mg_get_params(mg_handle h, mg_fparams* out);

/* ---- transfer (TransferToCL / TransferFromCL, host_CL.cpp:1608-1668) -------------------- */
mg_status mg_buffer_bytes(mg_handle h, int32_t buf_id, size_t* bytes);
mg_status mg_upload(mg_handle h, int32_t buf_id, const void* host, size_t bytes);
mg_status mg_download(mg_handle h, int32_t buf_id, void* host, size_t bytes);
/* Page-locked host buffers for mg_upload/mg_download (copies from them run at full link
 * bandwidth).  Convenience with no counterpart in the reference. */
/* One host exchange cycle with a single synchronisation: uploads `in`, runs nsteps steps with
 * `flags`, downloads `out` (same buffer ids, layouts and byte counts as mg_upload /
 * mg_download), all queued in order on the handle's stream.  For a host that exchanges state
 * every step (the reference's TransferToCL / Run / TransferFromCL cycle); pinned buffers from
 * mg_host_alloc give the full host-link bandwidth. */
typedef struct mg_io {
    int32_t buf_id;
    void* host;
    size_t bytes;
} mg_io;
mg_status mg_step_io(mg_handle h, const mg_io* in, uint32_t nin, uint32_t nsteps, uint32_t flags,
                     const mg_io* out, uint32_t nout);
mg_status mg_host_alloc(size_t bytes, void** out);
mg_status mg_host_free(void* ptr);
/* mNumPoints (particles in the grid after the last sort) and mActivePoints. */
mg_status mg_get_counts(mg_handle h, uint32_t* num_points, uint32_t* active_points);

/* ---- stages (the *CL wrappers of host_CL.cpp / host_CUDA.cpp) --------------------------- */
mg_status mg_insert_particles(mg_handle h);     /* InsertParticlesCL, host_CL.cpp:228-426 */
mg_status mg_prefix_sum_cells(mg_handle h);     /* PrefixSumCellsCL, host_CL.cpp:429-863 */
mg_status mg_counting_sort_full(mg_handle h);   /* CountingSortFullCL, host_CL.cpp:1064-1413 */
mg_status mg_compute_pressure(mg_handle h);     /* ComputePressureCL, host_CL.cpp:1918 */
mg_status mg_compute_force(mg_handle h);        /* ComputeForceCL, host_CL.cpp:1950 */
mg_status mg_compute_diffusion(mg_handle h);    /* ComputeDiffusionCL, host_CL.cpp:1936 */
mg_status mg_compute_genes(mg_handle h);        /* ComputeGenesCL, host_CL.cpp:1965-2019 */
mg_status mg_advance(mg_handle h);              /* AdvanceCL + AdvanceTime, host_CL.cpp:2182 */

/* ---- run loop (fluid_system.cpp:1919-2014) ---------------------------------------------- */
mg_status mg_run_physical_sort(mg_handle h);        /* Run2PhysicalSort */
mg_status mg_run_inner_physical_loop(mg_handle h);  /* Run2InnerPhysicalLoop */
mg_status mg_run_gene_action(mg_handle h);          /* Run2GeneAction */
/* Run2Remodelling (fluid_system.cpp:2037): re-forms broken bonds on the sorted state, after a
 * force pass and before integration.  Deterministic restatement of heal's bond-0 rule
 * (fluid_system_cuda.cu:1938-1975, 2047-2105, makeBond :1573-1593): each particle with a broken
 * bond proposes, for its lowest broken slot, the nearest particle within h that is not a
 * boundary marker, not already its partner and has a free incoming slot (ties: lower index);
 * proposals are accepted in (distance, index) order; the new bond has rest length = distance,
 * elastic limit 1.5 x rest length, the broken slot's modulus and damping. */
mg_status mg_run_remodelling(mg_handle h);
/* ComputeBondChangesCL(steps_per_InnerPhysicalLoop) (host_CUDA.cpp:744-761, kernel
 * computeBondChanges fluid_system_cuda.cu:1065-1331) over the living particles (gene 2): bonds
 * with rest length > 0 average their strain integrators over the steps, zero them, and scale
 * rest length and modulus by the genome's shifted tanh (tanh_param of the bond type the tissue
 * genes give); the first bond with rest length 0 or no partner gets change word 1 (heal) and
 * ends the particle's loop.  Until the next sort, mg_run_remodelling heals those slots, and the
 * change-list buffers (FBIN_COUNT_CHANGES, FBIN_OFFSET_CHANGES [9][cells],
 * FDENSE_LIST_LENGTHS_CHANGES [9], FDENSE_LISTS_CHANGES [9][2][N]: particle row then bond
 * row) download what PrefixSumChangesCL / CountingSortChangesCL (cuda:406-618) build. */
mg_status mg_compute_bond_changes(mg_handle h, uint32_t steps_per_inner_loop);
/* Run2Remodelling(steps_per_InnerPhysicalLoop) (fluid_system.cpp:2037-2071): computeBondChanges,
 * then heal of the slots it flagged. */
mg_status mg_run_remodelling_steps(mg_handle h, uint32_t steps_per_inner_loop);
/* ZeroVelCL (host_CUDA.cpp:851-857): velocity and evaluated velocity of every particle set to 0
 * (the freeze phase removes kinetic energy after each sort).  The reference's memset covers
 * mMaxPoints 32-bit words, a quarter of the float4 buffers; here all of them are cleared. */
mg_status mg_zero_vel(mg_handle h);
/* m_Time: the simulation time after the steps issued so far (AdvanceTime, fluid_system.cpp:2016) */
mg_status mg_get_time(mg_handle h, float* time);
/* nsteps full steps in the legacy Run() order (fluid_system.cpp:1179-1349), one sort per
 * step: insert, scan, sort, pressure, force, diffusion, genes, [remodel], advance, time. */
mg_status mg_step(mg_handle h, uint32_t nsteps, uint32_t flags);
mg_status mg_synchronize(mg_handle h);

/* ---- learned morphogen surrogate ------------------------------------------------------------
 * An MLP 48 -> 128 -> 128 -> 16 (GELU) maps a particle's 16 concentrations, the mean
 * concentrations of its diffusion neighbours and its 16 gene bits to the increment of one
 * morphogen stage (diffusion + gene reaction, computeDiffusion + computeGeneAction/tallyGene-
 * Action in the reference).  BF16 weights and activations, FP32 accumulation; trained with
 * Adam on (features, increment) pairs captured from plain steps.  In a step with
 * MG_STEP_SURROGATE the plain update still runs, as judge, for every judge_stride-th particle
 * every judge_period steps; a particle whose surrogate result is off by more than threshold
 * (relative) is handed to the plain method for the rest of the run. */
typedef struct mg_mlp_s* mg_mlp;
typedef struct mg_dataset_s* mg_dataset;
mg_status mg_mlp_create(uint64_t seed, mg_mlp* out);
mg_status mg_mlp_destroy(mg_mlp m);
/* Number of FP32 parameters (W1[128][48] b1 W2[128][128] b2 W3[16][128] b3, normalised
 * network) and of normalisation values (mu_x[48] 1/sd_x[48] mu_y[16] 1/sd_y[16]). */
mg_status mg_mlp_sizes(size_t* param_count, size_t* norm_count);
mg_status mg_mlp_get_params(mg_mlp m, float* host, size_t count);
mg_status mg_mlp_set_params(mg_mlp m, const float* host, size_t count);
mg_status mg_mlp_get_norm(mg_mlp m, float* host, size_t count);
mg_status mg_mlp_set_norm(mg_mlp m, const float* host, size_t count);
/* Forward + backward on n given rows (raw features x[n][48], increments y[n][16]): gradients
 * of the mean squared error of the normalised outputs, and the loss. */
mg_status mg_mlp_gradients(mg_mlp m, const float* x, const float* y, uint32_t n, float* grads,
                           double* loss);
/* Increments predicted by the in-step (tensor-memory) inference kernel for raw features. */
mg_status mg_mlp_infer(mg_mlp m, const float* x, uint32_t n, float* y);
mg_status mg_mlp_fit_normalization(mg_mlp m, mg_dataset d);
mg_status mg_mlp_train(mg_mlp m, mg_dataset d, uint32_t steps, uint32_t batch, float lr,
                       uint64_t seed, float* loss_curve);
mg_status mg_dataset_create(uint64_t capacity, mg_dataset* out);
mg_status mg_dataset_destroy(mg_dataset d);
/* Runs one plain step of h (flags: MG_STEP_PHYSICS or 0) and appends its particles'
 * (features, morphogen increment) pairs. */
mg_status mg_dataset_capture(mg_dataset d, mg_handle h, uint32_t flags);
mg_status mg_dataset_size(mg_dataset d, uint64_t* n);
mg_status mg_dataset_read(mg_dataset d, uint64_t first, uint32_t n, float* x, float* y);
/* Attaches a network to a simulation (NULL detaches); the network must outlive the use. */
mg_status mg_set_surrogate(mg_handle h, mg_mlp m, uint32_t judge_period, uint32_t judge_stride,
                           float threshold);
/* Particles judged, particles handed to the plain method, worst relative error seen. */
mg_status mg_surrogate_stats(mg_handle h, uint64_t* judged, uint64_t* handed_over, float* worst,
                             int32_t reset);

/* ---- tuning ------------------------------------------------------------------------------ */
enum mg_option {
    /* neighbour search of the density/diffusion pass: 0 = one thread walks its 27 cells
     * (the reference loop), 1 = warp-cooperative search (default), 2 = per-lane walk of the
     * 2x2x2 sub-cells within the radius (needs gsrch 3).  Results are identical. */
    MG_OPT_NEIGHBOR_SEARCH = 1,
    /* parameters of a healed bond: 0 = rest length = current distance, elastic limit 1.5 x rest
     * length, modulus and damping kept from the slot (default); 1 = makeBond's elastin defaults
     * from the genome (param[0]: elastLim, default rest length, modulus, damping,
     * fluid_system_cuda.cu:1573-1593) */
    MG_OPT_HEAL_PARAMS = 2,
    /* layout of FCONC in mg_upload / mg_download / mg_step_io: 0 = float[N][16], the rows the
     * kernels read (FCONC[p*16+tf], fluid_system_cuda.cu:739, 3097; default); 1 = float[16][N],
     * the reference host's own buffer (getConc(tf) = FCONC + tf*mMaxPoints, fluid_system.h:574),
     * transposed on the device */
    MG_OPT_CONC_LAYOUT = 3,
    /* steps between re-origins (0 = never; default 64): the bond records and cold fields are
     * kept by each particle's origin slot so that the sort does not move them; a re-origin sort
     * renumbers the origins to the sorted order (one step that moves them), after which the
     * force pass reads a warp's bond records from contiguous slots.  The first step after an
     * upload of FPOS re-origins too.  Results are identical for every period. */
    MG_OPT_REORIGIN_PERIOD = 4
};
mg_status mg_set_option(mg_handle h, int32_t option, int32_t value);

/* ---- launch-shape autotuner ------------------------------------------------------------------ */
/* Launch shape of the density pass: {warps per block (4 or 8), search groups (0: a cell and the
 * next cell of its row, 1: one cell), sub-cell bits per axis of the processing order (1 or 2),
 * neighbour search (MG_OPT_NEIGHBOR_SEARCH: 0, 1 or 2; 2 needs sub-cell bits 1)}.
 * Results are identical for every choice. */
mg_status mg_get_tuning(mg_handle h, int32_t choice[4]);
mg_status mg_set_tuning(mg_handle h, const int32_t choice[4]);
/* Threads per block of the force pass (k_force and k_force_in), the gather (the sort's
 * permutation of the carried state) and integration: {force, gather, advance}, each 128, 256
 * (the default) or 512.  Results are identical for every choice. */
mg_status mg_get_block_sizes(mg_handle h, int32_t threads[3]);
mg_status mg_set_block_sizes(mg_handle h, const int32_t threads[3]);
/* Times every density-pass launch shape over `steps` plain steps (flags: physics/genes only)
 * on the handle's current state, restoring the state after each trial, and keeps the fastest
 * (the default shape unless another is more than 3% faster); then, with that shape, the block
 * sizes of the force, gather and advance passes one at a time, by the same rule (read them
 * with mg_get_block_sizes).  choice receives the density shape as mg_get_tuning gives it.
 * Needs a free device allocation the size of the handle's arena for the snapshot. */
mg_status mg_autotune(mg_handle h, uint32_t steps, uint32_t flags, int32_t choice[4],
                      float* ms_per_step);

/* ---- measurement ------------------------------------------------------------------------- */
/* Runs nsteps of mg_step and returns their device time (CUDA events on the handle's stream). */
mg_status mg_time_steps(mg_handle h, uint32_t nsteps, uint32_t flags, float* ms);
/* Per-kernel device time: when enabled, every stage kernel launch of mg_step is bracketed by
 * CUDA events; mg_profile_read returns, per kernel slot, launches and total milliseconds. */
mg_status mg_profile_enable(mg_handle h, int32_t enable);
mg_status mg_profile_read(mg_handle h, int32_t max_slots, char* names /* max_slots*32 */,
                          uint32_t* launches, double* total_ms, int32_t* nslots);
/* Algorithmic DRAM bytes per particle and per cell of one kernel slot (by name) or of the
 * whole step (name NULL), for the roofline. */
mg_status mg_algorithmic_bytes(mg_handle h, const char* kernel, uint32_t flags,
                               double* bytes_per_particle, double* bytes_per_cell);
/* Number of GPU kernels mg_step/mg_time_steps have launched on this handle. */
uint64_t mg_kernel_launches(mg_handle h);
/* Device memory of the handle: the arena made by mg_create, and everything it holds now
 * (arena, upload staging, dense gene lists and surrogate buffers once made). */
mg_status mg_device_bytes(mg_handle h, size_t* arena, size_t* total);

/* ---- files (fileCL_IO.cpp formats) ------------------------------------------------------------ */
/* SimParams.txt fields (ReadSimParams / WriteSimParams, fileCL_IO.cpp:471-600). */
typedef struct mg_simparams {
    float time, dt, simscale, grid_density, visc, surface_tension, rest_density, spacing, mass,
        radius, dist, smooth_radius, intstiff, extstiff, extdamp, accel_limit, vel_limit, grav,
        ground_slope, force_min, force_max, force_freq;
    float plane_grav_dir[3];
    float grid_size;
    float volmin[3], volmax[3], initmin[3], initmax[3];
} mg_simparams;
mg_status mg_read_simparams(const char* path, mg_simparams* out);
mg_status mg_write_simparams(const char* dir, const mg_simparams* sp); /* writes dir/SimParams.txt */
/* The set-up ReadPointsCSV2 performs before allocating (fileCL_IO.cpp:353-361): grid cell
 * 2 * smooth radius / grid density, SetupSpacing's density from spacing and particle bounds
 * (fluid_system.cpp:2521-2546), SetupGrid, gravity = plane direction * gravity
 * (UpdateParams, fluid_system.cpp:617).  gsrch_override 0 keeps SetupGrid's own gsrch. */
mg_status mg_fparams_from_simparams(const mg_simparams* sp, int32_t gsrch_override, mg_fparams* out);
/* genome.csv (ReadGenome / WriteGenome, fileCL_IO.cpp:71-249).  The reference's integer fields
 * are read as floats; integer_fields = 1 writes them as integers (the reference format, values
 * rounded), 0 writes the floats in the same layout. */
mg_status mg_read_genome(const char* path, mg_genome* out);
mg_status mg_write_genome(const char* dir, const mg_genome* g, int32_t integer_fields); /* dir/genome.csv */
/* Particle CSV of SavePointsCSV2 / ReadPointsCSV2 (fileCL_IO.cpp:250-469) over host arrays in
 * the mg_upload layouts (n particles; epigen is [16][n]).  Each CSV line holds one particle's
 * 16 concentrations.  conc is [n][16], the layout the kernels read (FCONC[p*16+tf], cuda:739,
 * 3097); conc_species_major = 1 takes conc as [16][n] instead, the reference host's getConc
 * layout (FCONC[tf*maxPoints+p], fluid_system.h:574) that SavePointsCSV2 indexes
 * (fileCL_IO.cpp:323-326), for hosts that keep their buffers that way. */
typedef struct mg_points {
    uint32_t n;
    float* pos;            /* [n][4] */
    float* vel;            /* [n][4] */
    uint32_t* age;         /* [n] */
    uint32_t* color;       /* [n] */
    uint32_t* elastidx;    /* [n][54] */
    uint32_t* particle_id; /* [n] */
    uint32_t* mass_radius; /* [n] mass | radius << 16 */
    uint32_t* nerve;       /* [n] */
    uint32_t* pidx;        /* [n][12] */
    float* conc;           /* [n][16], or [16][n] with conc_species_major */
    uint32_t* epigen;      /* [16][n] */
    uint32_t conc_species_major;
} mg_points;
mg_status mg_count_points_csv(const char* path, uint32_t* n); /* lines - 1 */
mg_status mg_read_points_csv(const char* path, mg_points* pts);
/* writes dir/particles_pos_vel_color%04d.csv with frame + 100000 (SavePointsCSV2's naming) */
mg_status mg_write_points_csv(const char* dir, int32_t frame, const mg_points* pts);

/* SpecificationFile.txt (ReadSpecificationFile / WriteSpecificationFile_fromLaunchParams,
 * fileCL_IO.cpp:742-879, 1006-1114): the run description of the reference's drivers.  Paths
 * are at most 255 characters without spaces (read with %s); the y/n switches are characters. */
typedef struct mg_spec {
    uint32_t num_particles, demo_type, sim_space;
    float time, dt, gridsize, spacing, simscale, smooth_radius, visc, surface_tension, mass, radius,
        intstiff, extstiff, extdamp, accel_limit, vel_limit, grav, ground_slope, force_min,
        force_max, force_freq;
    float dim[3], pos[3], volmin[3], volmax[3], initmin[3], initmax[3];
    char params_path[256], points_path[256], genome_path[256], out_path[256];
    uint32_t num_files, steps_per_inner_loop, steps_per_file, freeze_steps, debug, file_num;
    char save_ply, save_csv, save_vtp, gene_activity, remodelling, read_genome;
    float actuation_factor, actuation_period;
} mg_spec;
mg_status mg_read_specification(const char* dir, mg_spec* out);        /* dir/SpecificationFile.txt */
mg_status mg_write_specification(const char* dir, const mg_spec* spec); /* dir/SpecificationFile.txt */
/* results.csv (WriteResultsCSV, fileCL_IO.cpp:1117-1142): one line of run totals.  timesteps =
 * (num_files / 100) * steps_per_inner_loop * steps_per_file of spec; num_bonds_end counts the
 * bonds of elastidx ([n][54], the FELASTIDX layout) with rest length > 0; the reference writes
 * its 65535 marker for num_bonds_start, which the caller passes. */
mg_status mg_write_results_csv(const char* input_folder, const char* output_folder,
                               const mg_spec* spec, uint32_t num_particles_start,
                               uint32_t num_particles_end, uint32_t num_bonds_start,
                               const uint32_t* elastidx, uint32_t n);
/* VTK XML PolyData (ASCII) of a sorted state, SavePointsVTP2's content (fileCL_IO.cpp:1223-1655)
 * written without VTK: the first `active` particles and the 8 corners of [volmin, volmax] as
 * points; per particle 6 lines, one per bond slot, to its partner (to itself when the slot has
 * no partner or a rest length below 1e-6), and 6 self-lines per corner, so the bond arrays
 * (cell data: parent index, parent id, partner index, partner id, slot, 0; elastic limit, rest
 * length, modulus, damping, both strain integrators) have one tuple per line; point data FAGE,
 * FCLR, FPARTICLE_ID, FMASS_RADIUS (mass, radius), FNERVEIDX, FVEL, FVEVAL, FFORCE, FPRESS,
 * "FDENSITY,(1/density,density)", FCONC_0..15, FEPIGEN_0..15, F_TISSUE_TYPE.  The reference
 * builds the line cells but no longer attaches them; here they are written.  File:
 * dir/particles_pos_vel_color%04d.vtp with frame + 100000.  veval, force: [n][4]; press,
 * invdens: [n] (FDENSITY holds 1/density). */
mg_status mg_write_points_vtp(const char* dir, int32_t frame, const mg_points* pts, uint32_t active,
                              const float* veval, const float* force, const float* press,
                              const float* invdens, const float volmin[3], const float volmax[3]);

/* ---- packed instances (parameter sweeps in one system) ------------------------------------------
 * n_inst independent tissues advanced as one system: every stage is one kernel launch over all
 * instances' particles.  Instance k keeps its own parameters' box, grid (origin, resolution;
 * the cell size is shared), intstiff and genome, and its own coordinate frame, so each instance
 * evaluates exactly what it evaluates as a system of its own (same bits); the other
 * parameters must be equal.  Its cells are a slab of a shared grid (slabs stacked along y), so
 * after each sort its particles are one contiguous segment of the sorted order
 * (mg_instance_ranges).  Buffers are exchanged like a single system of sum(max_points)
 * particles: instance 0's particles first, bond partners and incoming-bond entries as indices
 * into that concatenation; FGCELL / FBIN_* refer to the shared grid.  Steps take
 * MG_STEP_PHYSICS / GENES / FREEZE (no surrogate, remodelling or special particles);
 * parameters and genomes are fixed at creation.  The reference runs a sweep as separate jobs
 * (src/slurm/Morphogenesis_param_sweep.slurm; axes in src/SpecfileBatchGenerator.cpp:87-192). */
mg_status mg_create_packed(const mg_fparams* params, const mg_genome* genomes,
                           const uint32_t* max_points, uint32_t n_inst, mg_handle* out);
/* Sorted-index segment [first[k], first[k] + count[k]) of instance k after the last sort. */
mg_status mg_instance_ranges(mg_handle h, uint32_t* first, uint32_t* count);

/* ---- batched instances (parameter sweeps) --------------------------------------------------- */
/* A batch steps many independent systems together (each keeps its own particles, grid,
 * parameters and genome): one CUDA graph launch per step advances every member, the members'
 * kernels running concurrently.  Members must live on one device, must not be profiling, and
 * must outlive the batch; their own streams wait for the batch's steps.  Changes to a member's
 * parameters, genome or options apply from the next batch step (its steps are captured anew). */
typedef struct mg_batch_s* mg_batch;
mg_status mg_batch_create(const mg_handle* members, uint32_t count, mg_batch* out);
mg_status mg_batch_destroy(mg_batch b);
mg_status mg_batch_step(mg_batch b, uint32_t nsteps, uint32_t flags);
/* nsteps batch steps, device time of the whole run (CUDA events on the batch stream) */
mg_status mg_batch_time_steps(mg_batch b, uint32_t nsteps, uint32_t flags, float* ms);

/* ---- failure-detection self-test (no counterpart in the reference) ------------------------- */
/* Runs one bounded device-side wait against a flag that nothing sets, on buffers of its own,
 * and reports whether the wait gave up as designed.  which = 0: the prefix sum's look-back
 * (a scan whose first tile is never launched); which = 1: the surrogate inference's
 * tensor-core completion wait (an inference CTA whose MMAs are withheld; the CTA then frees
 * its tensor memory); which = 2: the training GEMM's completion wait (a GEMM CTA whose MMAs are
 * withheld; mg_mlp_train and mg_mlp_gradients return MG_ERR_DEVICE_TIMEOUT when such a wait
 * runs out).  spin_limit: polls before giving up (1 .. 1048576).  Returns
 * MG_ERR_DEVICE_TIMEOUT when the wait gave up (the expected result, the same status a step
 * returns when one of these waits runs out), MG_OK if it did not, MG_ERR_CUDA on a CUDA error.
 * The CUDA context stays usable either way.  Uses the current device and synchronises. */
mg_status mg_selftest_bounded_wait(int32_t which, uint32_t spin_limit);

/* ---- allocation-free prefix sum (no counterpart in the reference) ------------------------ */
/* Largest n mg_prefix_sum_noalloc accepts: 16384 tiles of 4096 elements. */
#define MG_NOALLOC_SCAN_MAX 67108864ull
/* Exclusive prefix sum offsets[i] = counts[0] + ... + counts[i-1] (mod 2^32), the scan
 * mg_prefix_sum_cells runs, over the caller's own device arrays, for callers that may not
 * allocate device memory at that point (an application whose own pool owns all device memory,
 * code inside an allocator callback, a loop that cannot take cudaFree's device-wide
 * synchronisation).  It calls no allocating routine (a rejected call only records its error
 * text): its scratch is a fixed 128 KiB device array per device inside the library, which it
 * clears on the stream before each scan.
 *   counts, offsets  device arrays of n uint32 (must not overlap)
 *   n                0 .. MG_NOALLOC_SCAN_MAX; larger n is rejected with MG_ERR_INVALID_ARG
 *   total            optional device uint32 receiving the sum of all n counts
 *   error            optional device uint32 the caller has zeroed; bit 0 is set if a bounded
 *                    look-back wait gave up (the offsets are then invalid).  With error NULL such
 *                    a timeout goes unreported: the call still returns MG_OK (it does not wait for
 *                    the scan), so pass an error word wherever a timeout must be detected
 *   stream           a cudaStream_t passed as void* (NULL: the default stream); the call is
 *                    asynchronous on it and uses the current device
 * Every call looks up the scratch's address on the current device (cudaGetSymbolAddress, a
 * host-side lookup that allocates nothing, so a device reset cannot leave a stale address);
 * a device's first call may load the library's device code, so make that first call, with
 * the device current, before any stream capture begins.  Calls on one device
 * share the scratch: calls whose scans can overlap in time (different streams without
 * ordering, or several host threads at once) race and give wrong offsets; order them. */
mg_status mg_prefix_sum_noalloc(const uint32_t* counts, uint32_t* offsets, uint64_t n,
                                uint32_t* total, uint32_t* error, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MG_ABI_H */
