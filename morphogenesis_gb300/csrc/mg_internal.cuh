// mg_internal.cuh - device-side data layout and kernel interfaces of the GB300 pipeline.
//
// HBM layout (structure of arrays, one "carried" set per sort direction):
//   pos/vel/veval   float4[N]            (the reference's cl_float3 is 16 bytes too)
//   bond            uint4[6][N][2]       per bond slot a, particle p: two 16-byte words
//                     A = (partner, restlen, modulus, damping)
//                     B = (elastlim, partner particle ID, strain^2 integrator, strain integrator)
//                   i.e. FELASTIDX words (0,2,3,4 | 1,5,6,7); word 8 (change type) is cold.
//                   The force kernel's gather of incoming bonds reads A and B.x of the
//                   partner's record while the owner writes only B.z/B.w.
//   pidx            uint32[N][12]        FPARTICLEIDX, the reference layout
//   conc            float[N][16]         FCONC, the reference device layout
//   genes           uint32[N]            bit g set <=> FEPIGEN[g][p] != 0; bit 31: the particle's
//                                        morphogen update was handed to the plain method
//   origin          uint32[N]            slot of this particle in the cold arrays
// Cold arrays (indexed by origin, never permuted): FAGE, FCOLOR, FPARTICLE_ID, FMASS_RADIUS,
// FNERVEIDX and FELASTIDX word 8.
// Per step: cell/arrival-rank/order/newidx/scell uint32[N], press/invdens float[N],
// force float4[N], brk uint32[N], count/offset uint32[cells].
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include "../../include/mg_abi.h"

namespace mg {

constexpr int NB = 6;
constexpr int NTF = 16;
constexpr int NG = 16;
constexpr uint32_t UNDEF = 0xFFFFFFFFu;
constexpr uint32_t NO_PARTNER = 0xFFFFFFFFu;
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;                      // per thread
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS; // 4096 cells per tile
// The step's scans take 64 items per thread (16,384 cells per tile): with every tile of the
// grid in flight at once, a tile's look-back reads its predecessors' status 32 at a time until
// it meets an inclusive prefix, so fewer, larger tiles shorten the longest look-back.
constexpr int WIDE_SCAN_ITEMS = 64;
constexpr int WARP_CELL_MAX = 256;   // cells up to this size are ordered by one warp
constexpr int BLOCK_CELL_MAX = 8192; // up to this by one block in shared memory
constexpr uint32_t BIG_LIST_CAP = 1u << 16;
constexpr uint32_t SPIN_LIMIT = 1u << 22; // bounded look-back polls
#ifndef MG_NL_CAP
#define MG_NL_CAP 56
#endif
constexpr int NL_CAP = MG_NL_CAP;  // per-lane neighbour list of the warp-cooperative density pass
constexpr int FL_CAP = 32;  // fluid-force neighbours (dsq < 1) recorded per particle
constexpr int MLP_FEATURES = 48;
constexpr int PROP_K = 8;  // proposals a particle keeps for ranking (more: it walks its window)  // surrogate inputs: conc[16], neighbour-mean conc[16], gene bits[16]

// Error bits in the device error word.
enum : uint32_t {
    ERR_SCAN_TIMEOUT = 1u << 0,
    ERR_BIG_LIST_OVERFLOW = 1u << 1,
    ERR_EPIGEN_VALUE = 1u << 2,
    ERR_INDEX = 1u << 3,  // a data-dependent index past its buffer (bounds-checking builds)
};

#ifndef MG_BOUNDS_CHECK
#define MG_BOUNDS_CHECK 0
#endif

// Simulation parameters passed by value to every kernel (constant bank).
// Packed instances (independent tissues advanced as one system, mg_create_packed): the frame
// and the per-instance physics of instance k.  Every instance keeps its own coordinates and its
// own grid geometry (origin, cell size, resolution, scan limits); its cells are placed in a
// slab of the shared grid starting at row y = ybase, with the same x and z indices, so that its
// particles sort into one contiguous segment and every kernel evaluates exactly the
// expressions it evaluates for the instance alone.
struct InstParams {
    float gmin[3], gdelta[3], gcell[3];
    int res[3], scanmax[3];
    int ybase;
    float frame_y;  // y of the shared grid's row 0 in this instance's frame (gmin.y - ybase * cell)
    float istiff;
    float bmin[3], bmax[3];
};

// Largest block of the one-particle-per-thread passes the launch shape may pick.
constexpr int MG_PLAIN_MAX_THREADS = 512;

struct DevParams {
    float gmin[3], gdelta[3];
    float gcell[3];  // 1 / gdelta: a grid cell's extent per axis
    int res[3], scanmax[3];
    int adjcnt, nadj, gsrch;
    int adj[64];
    float sr, r2, r2diff, d2, pmass, rest, istiff, wc2, surf;
    // 1 / sr when sr is a power of two (then r / sr == r * (1 / sr) exactly), else 0
    float sr_inv_exact;
    // 1.0, read at run time: a unit multiplier the compiler cannot fold (the packed diffusion
    // sums are written as p * unit + nc so that they are not fused with the product p)
    float unit;
    float pr, bmin[3], bmax[3], estiff, damp, xmin_stiff, xmax_stiff, slope, one_minus_slope;
    float grav[3], AL, AL2, VL, VL2, vl_factor, dt;
    float actuation_factor, actuation_period;
    float null_z;
    int freeze;
    int uniform_diff;  // all 16 diffusion rates equal and nonzero (set from the genome)
    // launch-shape choices of the density pass (results do not depend on them; mg_autotune
    // picks them by timing): warps per block, search groups (0: a cell and the next cell of
    // its row, 1: one cell), sub-cell bits per axis of the processing order (1 or 2)
    int dens_warps, group_mode, sub_bits;
    // threads per block of the one-particle-per-thread passes (128, 256 or 512; mg_autotune
    // picks them by timing): force (k_force and k_force_in), gather, advance
    int force_threads, gather_threads, advance_threads;
    int full_epi;  // per-gene FEPIGEN words carried (countdowns, activation lists) instead of bits
    int heal_params;  // healed bonds: 0 rest length = distance (D5), 1 makeBond's genome defaults
    uint32_t cap;
    uint32_t cells;
    // packed instances (null / 0 for a single system): per-instance frames and physics,
    // per-instance genomes
    const InstParams* inst;
    const struct DevGenome* genomes;
    int n_inst;
    uint32_t* err;  // the device error word (where bounds-checking builds record ERR_INDEX)
};

// Bounds-checking builds (MG_BOUNDS_CHECK=1): a data-dependent index at or past its bound sets
// ERR_INDEX in the error word and is replaced by one inside the buffer, so the access stays in
// bounds and the host reports the error after the step.  Other builds return the index as it is.
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t checked(const DevParams& P, uint32_t i, uint32_t bound) {
#if MG_BOUNDS_CHECK
    if (i >= bound) {
        if (P.err) atomicOr(P.err, (uint32_t)ERR_INDEX);
        return bound ? bound - 1u : 0u;
    }
#endif
    (void)P;
    (void)bound;
    return i;
}
#endif

// Genome in device memory (float-widened, compacted sparse lists).
struct DevGenome {
    float sens[NG][NTF];
    float diff[NTF];
    float breakdown[NTF];
    int nsec[NG];
    int sec_tf[NG][NTF];
    float sec_rate[NG][NTF];
    int nact[NG];
    int act_gene[NG][NG];
    float act_thr[NG][NG];
    uint32_t delay[NG];
    float tanh_p[3][8];   // bond remodelling tanh parameters per bond type (l_a..l_d, s_a..s_d)
    float bparam[3][12];  // bond parameters per bond type (elastLim = 8, default rest length,
                          // modulus, damping = 9, 10, 11)
    int uniform;          // all 16 diffusion rates equal and nonzero
};

// Bond records are kept by particle origin (the slot a particle was uploaded to), not in sorted
// order, so the sort does not move them: per bond slot two [cap] arrays of uint4, the A half
// (-, rest length, modulus, damping) and the B half (elastic limit, partner's particle id,
// strain^2 integrator, strain integrator), and one [cap] array of partners, each the partner's
// current sorted index (the sort remaps it in place).  The force pass rewrites the integrators
// every step; with the halves in separate arrays its writes dirty the B sectors only.
// o: the particle's origin.
__host__ __device__ __forceinline__ size_t bond_ia(uint32_t cap, int a, uint32_t o) {
    return (size_t)(2 * a) * cap + o;
}
__host__ __device__ __forceinline__ size_t bond_ib(uint32_t cap, int a, uint32_t o) {
    return (size_t)(2 * a + 1) * cap + o;
}
__host__ __device__ __forceinline__ size_t bond_ip(uint32_t cap, int a, uint32_t o) {
    return (size_t)a * cap + o;
}

struct Carried {
    float4* pos;
    float4* vel;
    float4* veval;
    // bond records by origin (bond_ia / bond_ib / bond_ip), shared by both sets: the sort moves
    // only the origins and remaps the partners in place
    uint4* bond;        // [NB][2][cap]: per bond slot, the A halves then the B halves
    uint32_t* partner;  // [NB][cap]: the partner's sorted index (NO_PARTNER: none)
    uint32_t* pidx;
    float* conc;
    uint32_t* genes;
    uint32_t* origin;
    uint32_t* epi;  // [16][cap] FEPIGEN words when the full epigenetic state is kept, else null
    uint32_t* iid;  // packed instances: the particle's instance (UNDEF for parked slots), else null
    // pressure and 1/density: written by the density pass; a sort permutes them (and zeroes
    // the forces) as countingSortFull does, when the step does not compute them again
    float* press;
    float* invdens;
};

// Everything kept by origin: the cold fields and the bond records (the carried sets' bond and
// partner pointers are this space's).
struct Cold {
    uint32_t* age;
    uint32_t* color;
    uint32_t* pid;
    uint32_t* mass_radius;
    uint32_t* nerve;
    uint32_t* change;  // [cap][NB]
    uint4* bond;        // [NB][2][cap] (bond_ia / bond_ib)
    uint32_t* partner;  // [NB][cap] (bond_ip)
};

struct Scratch {
    uint32_t* cell;     // unsorted cell of particle i (UNDEF outside the window)
    uint32_t* arank;    // arrival rank within the cell (not deterministic)
    uint32_t* order;    // arrival order: order[offset[cell] + arank[i]] = i (not stable)
    unsigned long long* okey;  // the same slots' keys (sub-cell code << 32 | i)
    uint32_t* sorted;   // sorted[p] = pre-sort index of the particle sorted to p (stable)
    uint32_t* work;     // density-pass processing order: sorted slots, cell by cell, each
                        // cell's particles by sub-cell Morton code (a permutation of [0, nactive))
    uint8_t* sub;       // Morton code of particle i's sub-cell inside its cell
    unsigned long long* subcnt;  // [cells] with 2x2x2 sub-cells: count of each sub-cell code
                                 // (8 bits each) of cells below WARP_CELL_MAX particles
    uint32_t* newidx;   // newidx[i] = sorted index of pre-sort particle i (UNDEF if dropped)
    uint32_t* scell;    // cell of sorted particle p
    float4* force;
    float4* bterm;      // [NB][cap] each own bond's acceleration on its partner in the last force
                        // pass (x, y, z; w = the partner's index bits, UNDEF when not evaluated)
    uint32_t* brk;      // bonds that broke in the last force pass
    uint32_t* flist;    // [FL_CAP][cap] fluid-force neighbours found by the density pass
    uint32_t* fcount;   // [cap] their number (> FL_CAP: search again)
    uint32_t* count;    // [cells]
    uint32_t* offset;   // [cells]
    unsigned long long* scan_status;  // [tiles]
    uint32_t* counters; // [0] scan tile ticket, [1] big-cell list length, [2] error word,
                        // [3] nactive, [5] step counter (incremented by insert),
                        // [6] density-pass overflow queue length, [7], [8] simulation time
                        // (float bits, slot = step counter parity)
    uint32_t* ovf;      // [cap] particles whose neighbours overflow a lane's list
    uint8_t* freemask;  // [cap] remodelling: free incoming slots
    uint32_t* prop_cnt;   // [cap] remodelling: proposals received
    uint32_t* prop_list;  // [cap][PROP_K] remodelling: the first PROP_K proposers
    uint32_t* prop;     // [cap] remodelling: proposed partner
    float* propd;       // [cap] remodelling: its squared distance
    uint32_t* big_list; // [BIG_LIST_CAP] cells that need the block-level ordering
};

// ---- launchers (all on one stream; no host synchronisation inside) ----------------------
cudaError_t physics_init();  // per-kernel attributes, once per device before the first launch
// warp_order: sub-cell codes ordered for the warp-cooperative searches (x-first slabs); false
// gives the Morton codes the per-lane fine-cell search reads as positions
void launch_clear_bins(const DevParams& P, const Scratch& s, int num_sms, cudaStream_t st);
void launch_insert(const DevParams& P, const Carried& cur, const Scratch& s, bool warp_order,
                   cudaStream_t st);
// narrow: tiles of SCAN_TILE cells (the allocation-free scan's fixed scratch is sized for
// them), else of SCAN_THREADS * WIDE_SCAN_ITEMS
void launch_scan(const uint32_t* in, uint32_t* out, uint32_t n, unsigned long long* status,
                 uint32_t* ticket, uint32_t* total, uint32_t* err, cudaStream_t st,
                 bool narrow = false);
// status words of a scan of n cells (of the narrow tiles: enough for either)
size_t scan_status_words(uint32_t n);
// failure-detection self-tests: a bounded wait on a flag nothing sets (see the definitions)
cudaError_t scan_selftest_wait_timeout(uint32_t spin_limit, uint32_t* err_bits, cudaStream_t st);
void launch_place(const DevParams& P, const Scratch& s, cudaStream_t st);
// subcounts: also count each cell's 2x2x2 sub-cells (for the per-lane fine-cell search)
void launch_cellsort(const DevParams& P, const Scratch& s, int num_sms, bool subcounts,
                     cudaStream_t st);
// parts of the carried state a gather moves (the three make the whole state): positions,
// bonds, genes, origins and cells; concentrations; velocities and the incoming-bond table
// GATHER_REORIGIN (with GATHER_CORE): the particles' origins become their sorted indices,
// their cold fields and bond records move from space `cs` to space `cd` accordingly.
// GATHER_SCRATCH: pressure and 1/density moved with the particles and the forces zeroed, as
// countingSortFull does (cuda:219-221); steps whose density and force passes rewrite them skip it.
enum : int { GATHER_CORE = 1, GATHER_CONC = 2, GATHER_MOTION = 4, GATHER_ALL = 7, GATHER_REORIGIN = 8,
             GATHER_SCRATCH = 16 };
void launch_gather(const DevParams& P, const Carried& src, const float* src_conc,
                   const Carried& dst, float* dst_conc, const Scratch& s, cudaStream_t st,
                   int parts = GATHER_ALL, const Cold* cs = nullptr, const Cold* cd = nullptr);
// flags: 1 density/pressure, 2 diffusion, 4 gene reaction
// flags: 1 density, 2 diffusion, 4 gene reaction, 8 surrogate features, 16 capture of
// training pairs, 32 judge (plain update of sampled / handed-over particles into conc_plain).
// search: 0 direct walk, 1 warp-cooperative, 2 per-lane fine cells, 3 warp-cooperative for
// positions that moved since the last sort (no window cell is skipped by its geometric box).
// Optional outputs of the density pass besides pressure/density/concentrations.
// Surrogate inputs are scale-free: a particle's diffused and neighbour-mean concentrations are
// divided by its scale s = max_t |c_t| (after diffusion), and the network predicts the reaction
// increment divided by s.  The reaction is linear in the concentrations, so this keeps the
// relative error of the prediction independent of how far the concentrations have decayed.
struct DensExtra {
    __nv_bfloat16* feat;       // FEATURES: surrogate inputs [cap][48] bf16
    float* feat_scale;         // FEATURES: the particle's scale s [cap]
    float* cap_x;              // CAPTURE: dataset features [..][48] for particle 0 of this pass
    float* cap_y;              // CAPTURE: dataset targets (reaction increment / s) [..][16]
    float* conc_plain;         // JUDGE: plain update of judged / handed-over particles
    uint32_t* epi;             // full epigenetic state of the current set ([16][cap]) or null
    const uint32_t* step;      // JUDGE: device step counter
    uint32_t judge_period, judge_stride;
    // re-forming candidates: the neighbours within h of each particle, in canonical order,
    // indexed by the particle's position in the processing order ([NL_CAP][cap]), with their
    // number (0xFFFFFFFF: not recorded, the particle overflowed)
    uint32_t* hlist;
    uint32_t* hcount;
    const uint32_t* iid;       // packed instances: instance of each sorted particle, else null
};
// G: the genome in device memory; Gh: its host copy, passed by value to the warp search so
// its uniform reads go through the constant cache
void launch_dens(const DevParams& P, const DevGenome* G, const DevGenome& Gh, const Carried& cur, const float* conc_in,
                 float* conc_out, const Scratch& s, int flags, int search, int num_sms,
                 cudaStream_t st, const DensExtra* extra = nullptr);

// incoming_in_advance: the integration follows directly and adds the incoming-bond reactions
// itself (launch_advance with incoming), so k_force_in is not launched
void launch_force(const DevParams& P, const Carried& cur, const Scratch& s, bool use_list,
                  cudaStream_t st, bool incoming_in_advance = false);
void launch_apply_breaks(const DevParams& P, const Carried& cur, const Scratch& s, cudaStream_t st);
// re-forming of broken bonds on the sorted state, breaks already applied (D5)
// computeBondChanges over the living particles; steps = steps_per_InnerPhysicalLoop
void launch_bond_changes(const DevParams& P, const DevGenome* G, const Carried& cur,
                         const Cold& cold, const Scratch& s, float steps, cudaStream_t st);
// change lists from the bonds' change words: counts / offsets [9][cells], lists [9][2][cap]
void launch_change_cell_counts(const DevParams& P, const Carried& cur, const Cold& cold,
                               const Scratch& s, uint32_t* ccount, cudaStream_t st);
void launch_change_lists(const DevParams& P, const Carried& cur, const Cold& cold,
                         const Scratch& s, const uint32_t* coffset, uint32_t* lists,
                         cudaStream_t st);
// heal: from_changes takes the slots computeBondChanges flagged (change word bit 0), else the
// D5 rule (lowest slot with an active partner and a failed rest-length test).  prune: positions
// are those of the last sort, so window cells may be skipped by their geometric box
// hcount / hlist: the density pass's record of each particle's neighbours within h, taken
// instead of a new search (null: search)
void launch_remodel(const DevParams& P, const DevGenome* G, const Carried& cur, const Cold& cold,
                    const Scratch& s, bool from_changes, bool prune, const uint32_t* hcount,
                    const uint32_t* hlist, cudaStream_t st);
// special: externalActuation / fixedParticles for genes 12 / 11 (SpecialParticlesCL);
// incoming: add the incoming-bond reactions to the force first (after launch_force with
// incoming_in_advance)
void launch_advance(const DevParams& P, const Carried& cur, const Scratch& s, bool apply_breaks,
                    cudaStream_t st, bool special = false, bool incoming = false);

// ---- import/export between the reference layouts and the device layout -------------------
// FCONC rows [cap][16] <-> species-major [16][cap]
void launch_conc_transpose(uint32_t cap, const float* src, float* dst, bool to_species_major,
                           cudaStream_t st);
void launch_import_bonds(const DevParams& P, const uint32_t* ref, const Carried& cur,
                         const Cold& cold, cudaStream_t st);
void launch_export_bonds(const DevParams& P, const Carried& cur, const Cold& cold,
                         const Scratch& s, bool apply_breaks, uint32_t* ref, cudaStream_t st);
void launch_import_epigen(const DevParams& P, const uint32_t* ref, const Carried& cur,
                          uint32_t* err, cudaStream_t st);
void launch_export_epigen(const DevParams& P, const Carried& cur, const Scratch& s,
                          uint32_t* ref, cudaStream_t st);
void launch_import_cold(const DevParams& P, const uint32_t* ref, const Carried& cur,
                        uint32_t* cold_field, cudaStream_t st);
void launch_export_cold(const DevParams& P, const Carried& cur, const Scratch& s,
                        const uint32_t* cold_field, uint32_t null_value, uint32_t* ref,
                        cudaStream_t st);
// FGCELL / FGNDX / FBIN views.  mode 1: after insert (pre-sort indices), 2: after sort.
void launch_export_grid_index(const DevParams& P, const Scratch& s, int which, int mode,
                              uint32_t* ref, cudaStream_t st);
void launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st);
void launch_identity(uint32_t* p, uint32_t n, cudaStream_t st);
void launch_init_set(uint32_t cap, const Carried& c, cudaStream_t st);
// full epigenetic state: words from the gene bits (INT_MAX / 0), bits from the words
void launch_bits_to_words(uint32_t cap, const Carried& c, cudaStream_t st);
void launch_words_to_bits(uint32_t cap, const Carried& c, cudaStream_t st);
// dense per-gene lists from the sorted gene bits
void launch_gene_cell_counts(const DevParams& P, const Carried& cur, const Scratch& s,
                             uint32_t* gcount, cudaStream_t st);
void launch_gene_lists(const DevParams& P, const Carried& cur, const Scratch& s,
                       const uint32_t* goffset, uint32_t* lists, cudaStream_t st);

// Records the calling thread's error text (what mg_last_error(NULL) returns) and gives st back.
mg_status record_thread_error(mg_status st, const char* msg);

}  // namespace mg
