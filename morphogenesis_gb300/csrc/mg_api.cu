// mg_api.cu - the C-ABI (include/mg_abi.h): handle, device memory arena, transfers, stage
// entry points and the CUDA-graph-captured step.
//
// Reference host side replaced here: FluidSetupCL / FluidParamCL / UpdateGenome
// (host_CL.cpp:39-174, fluid_system.cpp:494-610), TransferToCL / TransferFromCL
// (host_CL.cpp:1608-1668), the *CL stage wrappers (host_CL.cpp:228-2264) and the Run2* loop
// (fluid_system.cpp:1919-2014).  Where the reference calls clFinish after every kernel and
// reads counts back to the host every sort, the whole step here is one CUDA graph with the
// active particle count kept on the device.
#include <nvtx3/nvToolsExt.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/mg_abi.h"
#include "mg_internal.cuh"
#include "mg_mlp.cuh"

#ifndef MG_BATCH_GROUP
#define MG_BATCH_GROUP 32
#endif

using namespace mg;

namespace {

thread_local std::string g_thread_error;

constexpr int PHASE_UNSORTED = 0, PHASE_INSERTED = 1, PHASE_SORTED = 2;

struct ProfSlot {
    std::string name;
    uint32_t launches = 0;
    double ms = 0.0;
};

struct ProfMark {
    int slot;
    cudaEvent_t a, b;
};

}  // namespace

struct mg_system {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    mg_fparams params{};
    mg_genome genome{};
    DevParams P{};
    DevGenome* dG = nullptr;
    DevGenome hG{};  // host copy of *dG (the warp density pass takes the genome as a parameter)
    // incremented whenever the captured steps go stale (parameters, genome, options): batches
    // that hold this handle's steps rebuild theirs
    uint64_t graph_epoch = 0;
    uint32_t cap = 0;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    Carried set[2]{};
    int cur = 0;
    int conc_cur = 0;
    Cold cold{};      // the current origin space (cold fields, bond records)
    Cold cold_alt{};  // the other one, which a re-origin moves the records into
    int osp = 0;      // which of the two is current (part of the captured graphs' keys)
    // re-origin: every `reorigin_period` plain steps (and at the first after an upload of
    // positions) the sort renumbers origins to the sorted order, so that the force pass reads
    // the bond records of a warp's particles from contiguous slots; 0 = never
    uint32_t reorigin_period = 64, since_reorigin = 0;
    bool reorigin_due = true;
    Scratch s{};
    void* staging = nullptr;
    size_t staging_bytes = 0;
    uint32_t* dense = nullptr;  // gcount | goffset | lists | lens (allocated on demand)
    uint32_t* changes = nullptr;  // change lists: ccount | coffset | lists | lens (on demand)
    bool changes_valid = false;   // computeBondChanges ran since the last sort (heal uses it)
    uint32_t* epi_mem = nullptr;  // full epigenetic state of both sets (allocated on demand)
    int phase = PHASE_UNSORTED;
    bool ever_sorted = false;
    bool brk_pending = false;
    bool flist_valid = false;   // fluid-force lists match the current positions and order
    bool drifted = false;       // positions changed since the last sort (cells no longer bound them)
    uint32_t* hmem = nullptr;   // re-forming candidates recorded by the density pass: count [cap]
                                // then list [NL_CAP][cap] (allocated with the first remodelling step)
    int search = 1;             // density pass search: 0 direct walk, 1 warp-cooperative
    int conc_species_major = 0; // FCONC exchanged as [16][N] (MG_OPT_CONC_LAYOUT 1)
    float time = 0.f;
    std::string err;
    std::map<uint64_t, cudaGraphExec_t> graphs;
    // steps with their host exchange overlapped (mg_step_io): graphs keyed by the step's flags,
    // buffer state and exchange list; side streams and fork / join events used in capture
    std::map<std::string, cudaGraphExec_t> io_graphs;
    cudaStream_t io_st[2] = {nullptr, nullptr};
    cudaEvent_t io_ev[7] = {};
    // the velocities / incoming-bond table of the last gather still to move (their upload was in
    // flight): moved after this event, before the force pass reads them
    cudaEvent_t motion_ready = nullptr;
    bool profile = false;
    std::vector<ProfSlot> prof;
    std::vector<ProfMark> marks;
    uint64_t launches = 0;  // kernels launched by mg_step (one graph step counts its kernels)
    // learned morphogen surrogate (attached network is borrowed, not owned)
    mg::Mlp* sur = nullptr;
    __nv_bfloat16* feat = nullptr;   // [cap][48] surrogate inputs
    CUtensorMap feat_map{};          // TMA view of feat for the inference kernel
    float* feat_scale = nullptr;     // [cap] per-particle scale of the inputs
    float* conc_plain = nullptr;     // [cap][16] plain update of judged / handed-over particles
    uint32_t* sur_stats = nullptr;   // [0] judged, [1] handed over, [2] worst relative error bits
    uint32_t judge_period = 10, judge_stride = 64;
    float judge_threshold = 1e-3f;
    // packed instances (mg_create_packed): per-instance frames, genomes and particle counts
    uint32_t n_inst = 0;
    InstParams* d_inst = nullptr;       // [n_inst] in the arena
    DevGenome* d_genomes = nullptr;     // [n_inst] in the arena
    std::vector<InstParams> inst;       // host copy
    std::vector<uint32_t> inst_count;   // particles per instance (slots in upload order)
};

struct mg_mlp_s {
    mg::Mlp m;
    cudaStream_t st;
};

// A batch of independent systems stepped together: one CUDA graph per (flags, buffer states)
// holds every member's captured step as an independent child graph, so one launch advances all
// members and the GPU runs their kernels concurrently.
struct mg_batch_s {
    std::vector<mg_system*> hs;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::map<std::string, cudaGraphExec_t> graphs;
    // members' capture epochs the cached graphs were made for: when one changes, every cached
    // graph holds stale parameters or genomes and is destroyed
    std::vector<uint64_t> epochs;
    std::string err;
};

struct mg_dataset_s {
    float* dx = nullptr;  // [capacity][48] raw features
    float* dy = nullptr;  // [capacity][16] morphogen increments
    uint64_t capacity = 0, size = 0;
};

namespace {

mg_status fail(mg_system* h, mg_status st, const std::string& msg) {
    if (h) h->err = msg;
    g_thread_error = msg;
    return st;
}

mg_status cuda_fail(mg_system* h, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(h, MG_ERR_CUDA, m);
}

#define MG_CUDA(h, expr)                                          \
    do {                                                          \
        cudaError_t e_ = (expr);                                  \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #expr);  \
    } while (0)

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Derived constants exactly as FluidParamCL (fluid_system.cpp:527-598) and FluidSetupCL
// (host_CL.cpp:39-106) compute them, in float.
void derive(DevParams& D, const mg_fparams& p, uint32_t cap) {
    std::memset(&D, 0, sizeof(D));
    for (int k = 0; k < 3; k++) {
        D.gmin[k] = p.grid_min[k];
        D.gdelta[k] = p.grid_delta[k];
        D.gcell[k] = 1.f / p.grid_delta[k];
        D.res[k] = p.grid_res[k];
        D.scanmax[k] = p.grid_res[k] - p.grid_srch;
        D.bmin[k] = p.pboundmin[k];
        D.bmax[k] = p.pboundmax[k];
        D.grav[k] = p.pgravity[k];
    }
    int c = 0;
    for (int y = 0; y < p.grid_srch; y++)
        for (int z = 0; z < p.grid_srch; z++)
            for (int x = 0; x < p.grid_srch; x++)
                if (c < 64) D.adj[c++] = (y * p.grid_res[2] + z) * p.grid_res[0] + x;
    D.adjcnt = p.grid_srch * p.grid_srch * p.grid_srch;
    D.nadj = (1 * p.grid_res[2] + 1) * p.grid_res[0] + 1;
    D.gsrch = p.grid_srch;
    D.sr = p.psmoothradius;
    {
        int ex = 0;
        const float m = std::frexp(p.psmoothradius, &ex);  // sr = m * 2^ex, m in [0.5, 1)
        D.sr_inv_exact = (m == 0.5f && std::isfinite(p.psmoothradius)) ? 1.0f / p.psmoothradius : 0.0f;
        D.unit = 1.0f;
    }
    D.r2 = p.psmoothradius * p.psmoothradius;
    D.d2 = p.psimscale * p.psimscale;
    D.r2diff = D.r2 / D.d2;  // computeDiffusion: r2 = fparam.r2 / d2 (cuda:3032)
    D.pmass = p.pmass;
    D.rest = p.prest_dens;
    D.istiff = p.pintstiff;
    D.wc2 = 21 / (2 * 3.141592f);
    D.surf = p.psurface_t;
    D.pr = p.pradius;
    D.estiff = p.pextstiff;
    D.damp = p.pdamp;
    D.xmin_stiff = (p.pforce_min + 1) * p.pextstiff;
    D.xmax_stiff = (p.pforce_max + 1) * p.pextstiff;
    D.slope = p.pground_slope;
    D.one_minus_slope = 1.0f - p.pground_slope;
    D.AL = p.paccel_limit;
    D.AL2 = p.paccel_limit * p.paccel_limit;
    D.VL = p.pvel_limit;
    D.VL2 = p.pvel_limit * p.pvel_limit;
    D.vl_factor = D.VL / sqrtf(D.VL2);
    D.dt = p.dt;
    D.actuation_factor = p.actuation_factor;
    D.actuation_period = p.actuation_period;
    D.null_z = p.pboundmin[2] - (float)(2 * p.grid_res[2]);
    D.freeze = p.freeze ? 1 : 0;
    D.cap = cap;
    D.dens_warps = 8;
    D.group_mode = 0;
    D.sub_bits = 2;
    D.force_threads = D.gather_threads = D.advance_threads = 256;
    D.cells = (uint32_t)p.grid_total;
}

mg_status check_params(mg_system* h, const mg_fparams* p) {
    if (!p) return fail(h, MG_ERR_INVALID_ARG, "params is NULL");
    if (p->grid_srch < 1 || p->grid_srch > 4)
        return fail(h, MG_ERR_INVALID_ARG, "grid_srch must be 1..4 (gridAdj holds 64 cells)");
    for (int k = 0; k < 3; k++)
        if (p->grid_res[k] <= p->grid_srch)
            return fail(h, MG_ERR_INVALID_ARG, "grid_res must exceed grid_srch on every axis");
    long long tot = (long long)p->grid_res[0] * p->grid_res[1] * p->grid_res[2];
    if (tot != p->grid_total || tot <= 0 || tot > 0x7fffffffLL)
        return fail(h, MG_ERR_INVALID_ARG, "grid_total must equal res.x*res.y*res.z (< 2^31)");
    if (!(p->psmoothradius > 0.f) || !(p->psimscale > 0.f) || !(p->pmass > 0.f))
        return fail(h, MG_ERR_INVALID_ARG, "psmoothradius, psimscale and pmass must be > 0");
    return MG_OK;
}

void clear_graphs(mg_system* h);

// Switches to the full epigenetic state: per-gene FEPIGEN words carried with the particles
// (countdowns and activation lists), initialised from the current gene bits.
mg_status enable_full_epi(mg_system* h) {
    if (h->P.full_epi) return MG_OK;
    if (h->P.n_inst)
        return fail(h, MG_ERR_UNSUPPORTED, "packed instances keep gene bits only (no FEPIGEN countdowns or activation lists)");
    const size_t words = (size_t)NG * h->cap;
    cudaError_t e = cudaMalloc(&h->epi_mem, 2 * words * sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        h->epi_mem = nullptr;
        return fail(h, MG_ERR_OOM, "full epigenetic state");
    }
    h->set[0].epi = h->epi_mem;
    h->set[1].epi = h->epi_mem + words;
    MG_CUDA(h, cudaMemsetAsync(h->epi_mem, 0, 2 * words * sizeof(uint32_t), h->stream));
    launch_bits_to_words(h->cap, h->set[h->cur], h->stream);
    h->P.full_epi = 1;
    clear_graphs(h);
    return MG_OK;
}

// The device form of a genome (rates and weights as float, sparse lists compacted); an empty
// string when it is valid, else the reason.
std::string make_dev_genome(const mg_genome& G, DevGenome& g) {
    std::memset(&g, 0, sizeof(g));
    for (int a = 0; a < NG; a++)
        for (int t = 0; t < NTF; t++) g.sens[a][t] = G.sensitivity[a][t];
    for (int t = 0; t < NTF; t++) {
        g.diff[t] = G.tf_diffusability[t];
        g.breakdown[t] = G.tf_breakdown_rate[t];
    }
    for (int a = 0; a < NG; a++) {
        int ns = (int)G.secrete[a][2 * NTF];
        if (ns < 0 || ns > NTF) return "secrete list count out of range";
        int k = 0;
        for (int j = 0; j < ns; j++) {
            int tf = (int)G.secrete[a][2 * j];
            if (tf < 0 || tf >= NTF) return "secrete list names a species out of range";
            g.sec_tf[a][k] = tf;
            g.sec_rate[a][k] = G.secrete[a][2 * j + 1];
            k++;
        }
        g.nsec[a] = k;
        // activation list (computeGeneAction cuda:752-757): entries naming a gene out of range
        // are skipped, at most 16 are read
        const int na = (int)G.activate[a][2 * NG];
        int m = 0;
        for (int j = 0; j < na && j < NG; j++) {
            const int og = (int)G.activate[a][2 * j];
            if (og < 0 || og >= NG) continue;
            g.act_gene[a][m] = og;
            g.act_thr[a][m] = G.activate[a][2 * j + 1];
            m++;
        }
        g.nact[a] = m;
        g.delay[a] = G.delay[a];
    }
    for (int t = 0; t < 3; t++) {
        for (int k = 0; k < 8; k++) g.tanh_p[t][k] = G.tanh_param[t][k];
        for (int k = 0; k < 12; k++) g.bparam[t][k] = G.param[t][k];
    }
    int uniform = g.diff[0] != 0.f;
    for (int t = 1; t < NTF; t++) uniform &= g.diff[t] == g.diff[0];
    g.uniform = uniform;
    return std::string();
}

bool has_activations(const DevGenome& g) {
    bool activations = false;
    for (int a = 0; a < NG; a++) activations |= g.nact[a] > 0;
    return activations;
}

mg_status upload_genome(mg_system* h) {
    DevGenome g;
    const std::string why = make_dev_genome(h->genome, g);
    if (!why.empty()) return fail(h, MG_ERR_INVALID_ARG, why);
    if (has_activations(g)) {  // activations change FEPIGEN words: keep the full state
        if (h->P.n_inst) return fail(h, MG_ERR_UNSUPPORTED, "packed instances take genomes without activation lists");
        mg_status st = enable_full_epi(h);
        if (st != MG_OK) return st;
    }
    if (h->P.uniform_diff != g.uniform) clear_graphs(h);
    h->P.uniform_diff = g.uniform;
    h->hG = g;
    clear_graphs(h);  // captured density launches hold the genome by value
    MG_CUDA(h, cudaMemcpyAsync(h->dG, &g, sizeof(g), cudaMemcpyHostToDevice, h->stream));
    MG_CUDA(h, cudaStreamSynchronize(h->stream));
    return MG_OK;
}

void clear_graphs(mg_system* h) {
    h->graph_epoch++;
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    for (auto& kv : h->io_graphs) cudaGraphExecDestroy(kv.second);
    h->io_graphs.clear();
}

uint32_t read_word(mg_system* h, const uint32_t* dptr, mg_status* st) {
    uint32_t v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, dptr, 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) *st = cuda_fail(h, e, "read device word");
    return v;
}

// Reads and clears the device error word; maps its bits to a status.
mg_status check_device(mg_system* h) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamSynchronize");
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, "kernel launch");
    mg_status st = MG_OK;
    uint32_t err = read_word(h, h->s.counters + 2, &st);
    if (st != MG_OK) return st;
    if (err == 0) return MG_OK;
    uint32_t zero = 0;
    cudaMemcpy(h->s.counters + 2, &zero, 4, cudaMemcpyHostToDevice);
    if (err & ERR_SCAN_TIMEOUT)
        return fail(h, MG_ERR_DEVICE_TIMEOUT, "prefix-sum look-back gave up waiting (bounded spin)");
    if (err & ERR_BIG_LIST_OVERFLOW)
        return fail(h, MG_ERR_GRID_OVERFLOW, "more than 65536 grid cells hold over 256 particles");
    if (err & mg::MLP_ERR_MBAR_TIMEOUT)
        return fail(h, MG_ERR_DEVICE_TIMEOUT, "surrogate inference: tensor-core completion wait gave up (bounded spin)");
    if (err & ERR_INDEX)
        return fail(h, MG_ERR_CUDA, "an index past its buffer (bounds-checking build): a kernel read a corrupt index");
    if (err & ERR_EPIGEN_VALUE)
        return fail(h, MG_ERR_UNSUPPORTED,
                    "FEPIGEN values other than 0 and INT_MAX (epigenetic countdowns) are not "
                    "supported by the GPU gene kernel");
    return fail(h, MG_ERR_CUDA, "unknown device error word");
}

// ---- profiling marks ------------------------------------------------------------------------
int prof_slot(mg_system* h, const char* name) {
    for (size_t k = 0; k < h->prof.size(); k++)
        if (h->prof[k].name == name) return (int)k;
    h->prof.push_back(ProfSlot{name, 0, 0.0});
    return (int)h->prof.size() - 1;
}

// An NVTX range around a host entry point or, in profiling mode, a stage's launches (named by
// the stage); a tool such as Nsight Systems or `ncu --nvtx` sees them, otherwise they cost a
// check of the NVTX dispatch table.
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

struct Mark {
    mg_system* h;
    bool on;
    ProfMark m{};
    Mark(mg_system* h_, bool on_, const char* name) : h(h_), on(on_) {
        if (!on) return;
        nvtxRangePushA(name);
        m.slot = prof_slot(h, name);
        cudaEventCreate(&m.a);
        cudaEventCreate(&m.b);
        cudaEventRecord(m.a, h->stream);
    }
    ~Mark() {
        if (!on) return;
        cudaEventRecord(m.b, h->stream);
        h->marks.push_back(m);
        nvtxRangePop();
    }
};

void prof_collect(mg_system* h) {
    cudaStreamSynchronize(h->stream);
    for (auto& m : h->marks) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, m.a, m.b);
        h->prof[m.slot].launches++;
        h->prof[m.slot].ms += ms;
        cudaEventDestroy(m.a);
        cudaEventDestroy(m.b);
    }
    h->marks.clear();
}

// ---- pipeline pieces -------------------------------------------------------------------------
float* conc_of(mg_system* h, int k) { return h->set[k].conc; }

void enqueue_insert_rank(mg_system* h, bool prof) {
    const DevParams& P = h->P;
    cudaStream_t st = h->stream;
    launch_clear_bins(P, h->s, h->num_sms, st);
    { Mark m(h, prof, "insert"); launch_insert(P, h->set[h->cur], h->s, h->search != 2, st); }
    { Mark m(h, prof, "scan"); launch_scan(h->s.count, h->s.offset, P.cells, h->s.scan_status,
                                           h->s.counters, h->s.counters + 3, h->s.counters + 2, st); }
    { Mark m(h, prof, "place"); launch_place(P, h->s, st); }
    { Mark m(h, prof, "cellsort"); launch_cellsort(P, h->s, h->num_sms, h->search == 2, st); }
}

// Internal step flag (never a caller's): this step's sort renumbers the origins.
constexpr uint32_t STEP_REORIGIN = 1u << 31;

// After a re-origin gather: the other origin space becomes the current one.
void swap_ospace(mg_system* h) {
    std::swap(h->cold, h->cold_alt);
    for (Carried& c : h->set) {
        c.bond = h->cold.bond;
        c.partner = h->cold.partner;
    }
    h->osp ^= 1;
}

// conc_ready / motion_ready: the concentrations / the velocities and incoming-bond table arrive
// later (uploads still in flight).  The rest is moved first, the concentrations after the
// stream has waited for conc_ready; the motion part is left to flush_motion, which the step
// calls before its force pass (nothing before it reads those fields).
// scratch: the step does not compute pressure, density and forces again after this sort, so
// the sort moves the first two and zeroes the forces as countingSortFull does.
void enqueue_gather(mg_system* h, bool prof, cudaEvent_t conc_ready = nullptr,
                    cudaEvent_t motion_ready = nullptr, bool reorigin = false, bool scratch = true) {
    int src = h->cur, dst = 1 - h->cur;
    int csrc = h->conc_cur, cdst = 1 - h->conc_cur;
    { Mark m(h, prof, "gather");
      const int first = GATHER_CORE | (conc_ready ? 0 : GATHER_CONC) | (motion_ready ? 0 : GATHER_MOTION) |
                        (reorigin ? GATHER_REORIGIN : 0) | (scratch ? GATHER_SCRATCH : 0);
      launch_gather(h->P, h->set[src], conc_of(h, csrc), h->set[dst], conc_of(h, cdst), h->s, h->stream, first,
                    &h->cold, &h->cold_alt);
      if (reorigin) swap_ospace(h);
      if (conc_ready) {
          cudaStreamWaitEvent(h->stream, conc_ready, 0);
          launch_gather(h->P, h->set[src], conc_of(h, csrc), h->set[dst], conc_of(h, cdst), h->s, h->stream,
                        GATHER_CONC);
      }
    }
    h->motion_ready = motion_ready;
    h->cur = dst;
    h->conc_cur = cdst;
    h->flist_valid = false;
    h->changes_valid = false;
    h->drifted = false;
}

// dens flags: 1 density, 2 diffusion, 4 genes.  Any conc-writing variant flips conc_cur.
void enqueue_dens(mg_system* h, int flags, bool prof, bool heal_list = false) {
    int cin = h->conc_cur, cout = 1 - h->conc_cur;
    DensExtra X{};
    if (heal_list) {
        X.hcount = h->hmem;
        X.hlist = h->hmem + h->cap;
    }
    { Mark m(h, prof, flags == 1 ? "pressure" : flags == 7 ? "density_diffusion_genes" : "diffusion_genes");
      launch_dens(h->P, h->dG, h->hG, h->set[h->cur], conc_of(h, cin), conc_of(h, cout), h->s, flags,
                  h->drifted && h->search ? 3 : h->search, h->num_sms, h->stream, &X); }
    if (flags & 6) h->conc_cur = cout;
    if (h->search && (flags & 3)) h->flist_valid = true;
}

// Host exchange folded into a step (mg_step_io): uploads before it, downloads after it, each a
// plain copy between a host buffer and a device buffer of the reference layout.
struct IoPlan {
    const mg_io* in = nullptr;
    uint32_t nin = 0;
    const mg_io* out = nullptr;
    uint32_t nout = 0;
};

// Device buffer that a plain copy exchanges with the host for buffer id (the mapping of
// mg_upload / mg_download for those ids), in the handle's current buffer state; null when the
// buffer needs a layout conversion.
void* direct_buffer(mg_system* h, int32_t id, bool upload) {
    Carried& c = h->set[h->cur];
    switch (id) {
    case MG_FPOS: return c.pos;
    case MG_FVEL: return c.vel;
    case MG_FVEVAL: return c.veval;
    case MG_FFORCE: return h->s.force;
    case MG_FPRESS: return c.press;
    case MG_FDENSITY: return c.invdens;
    case MG_FPARTICLEIDX: return c.pidx;
    case MG_FCONC: return h->conc_species_major ? nullptr : conc_of(h, h->conc_cur);
    case MG_FBIN_COUNT: return upload ? nullptr : h->s.count;
    case MG_FBIN_OFFSET: return upload ? nullptr : h->s.offset;
    default: return nullptr;
    }
}

// One step in the legacy Run() order (fluid_system.cpp:1179-1349), one sort per step.
// With an exchange plan (captured into the step's graph): FPOS is uploaded first on a side
// stream and the bin / scan / sort kernels start when it has arrived, while the other uploads
// continue on a second side stream that the gather waits for (the concentrations, uploaded
// last, are moved by a second gather kernel once they have arrived); FCONC is downloaded on a side
// stream as soon as the morphogen stage has written it, under the force and integration
// kernels; the other downloads follow the step, and the step ends when every copy has.
// Whether a step with these flags takes its re-forming candidates from the density pass: the
// pass runs the diffusion (or surrogate) neighbour sums at the positions the re-forming search
// sees, with a list-building search, and the record's memory exists.
bool heal_from_density(const mg_system* h, uint32_t flags) {
    return (flags & (MG_STEP_REMODEL | MG_STEP_BOND_CHANGES)) && (flags & (MG_STEP_GENES | MG_STEP_SURROGATE)) &&
           (h->search == 1 || h->search == 2) && h->hmem;
}

// Allocates the candidate record for a remodelling step (before any capture); without memory
// the step searches instead.
void prepare_step(mg_system* h, uint32_t flags) {
    if (!(flags & (MG_STEP_REMODEL | MG_STEP_BOND_CHANGES)) || h->hmem) return;
    if (cudaMalloc(&h->hmem, sizeof(uint32_t) * (size_t)h->cap * (1 + NL_CAP)) != cudaSuccess) {
        cudaGetLastError();
        h->hmem = nullptr;
    }
}

void enqueue_surrogate_morphogen(mg_system* h, bool density, bool prof, bool heal_list = false) {
    DensExtra X{};
    if (heal_list) {
        X.hcount = h->hmem;
        X.hlist = h->hmem + h->cap;
    }
    X.feat = h->feat;
    X.feat_scale = h->feat_scale;
    X.conc_plain = h->conc_plain;
    X.step = h->s.counters + 5;
    X.judge_period = h->judge_period;
    X.judge_stride = h->judge_stride;
    const int cin = h->conc_cur, cout = 1 - h->conc_cur;
    const int dflags = (density ? 1 : 0) | 2 | 4 | 8 | 32;
    { Mark m(h, prof, density ? "density_features" : "features");
      launch_dens(h->P, h->dG, h->hG, h->set[h->cur], conc_of(h, cin), conc_of(h, cout), h->s, dflags,
                  h->search, h->num_sms, h->stream, &X); }
    if (h->search) h->flist_valid = true;
    { Mark m(h, prof, "mlp_infer");
      // conc_out holds the diffused concentrations; the network adds the reaction increment
      launch_mlp_infer(h->sur, h->feat_map, h->feat_scale, conc_of(h, cout), h->conc_plain, conc_of(h, cout),
                       h->set[h->cur].genes, h->s.counters + 3, 0, h->s.counters + 5, h->judge_period,
                       h->judge_stride, h->judge_threshold, h->sur_stats, h->s.counters + 2,
                       h->num_sms, h->stream); }
    h->conc_cur = cout;
}

// The motion part of a gather whose upload was in flight (see enqueue_gather).
void flush_motion(mg_system* h, bool prof) {
    if (!h->motion_ready) return;
    Mark m(h, prof, "gather");
    cudaStreamWaitEvent(h->stream, h->motion_ready, 0);
    launch_gather(h->P, h->set[1 - h->cur], nullptr, h->set[h->cur], nullptr, h->s, h->stream, GATHER_MOTION);
    h->motion_ready = nullptr;
}

// Uploads the force pass reads first (the gather moves them last).
bool motion_buffer(int32_t id) { return id == MG_FVEL || id == MG_FVEVAL || id == MG_FPARTICLEIDX; }

void enqueue_step(mg_system* h, uint32_t flags, bool prof, const IoPlan* io = nullptr) {
    cudaStream_t st = h->stream;
    cudaStream_t A = io ? h->io_st[0] : nullptr, B = io ? h->io_st[1] : nullptr;
    cudaEvent_t* ev = h->io_ev;
    const bool up = io && io->nin;
    bool conc_up = false, motion_up = false;
    if (up) {
        cudaEventRecord(ev[0], st);
        cudaStreamWaitEvent(A, ev[0], 0);
        cudaStreamWaitEvent(B, ev[0], 0);
        // FPOS on A (the sort needs it first); on B the other buffers the gather's first part
        // moves, then FCONC (the density pass's input), then the velocities and the incoming-
        // bond table, which nothing reads before the force pass
        auto upload = [&](uint32_t k, cudaStream_t s) {
            cudaMemcpyAsync(direct_buffer(h, io->in[k].buf_id, true), io->in[k].host, io->in[k].bytes,
                            cudaMemcpyHostToDevice, s);
        };
        for (uint32_t k = 0; k < io->nin; k++)
            if (io->in[k].buf_id == MG_FPOS) upload(k, A);
        for (uint32_t k = 0; k < io->nin; k++)
            if (io->in[k].buf_id != MG_FPOS && io->in[k].buf_id != MG_FCONC && !motion_buffer(io->in[k].buf_id))
                upload(k, B);
        cudaEventRecord(ev[1], A);
        cudaEventRecord(ev[2], B);
        for (uint32_t k = 0; k < io->nin; k++)
            if (io->in[k].buf_id == MG_FCONC) {
                upload(k, B);
                conc_up = true;
            }
        if (conc_up) cudaEventRecord(ev[5], B);
        for (uint32_t k = 0; k < io->nin; k++)
            if (motion_buffer(io->in[k].buf_id)) {
                upload(k, B);
                motion_up = true;
            }
        if (motion_up) cudaEventRecord(ev[6], B);
        cudaStreamWaitEvent(st, ev[1], 0);
    }
    enqueue_insert_rank(h, prof);
    if (up) cudaStreamWaitEvent(st, ev[2], 0);
    enqueue_gather(h, prof, conc_up ? ev[5] : nullptr, motion_up ? ev[6] : nullptr,
                   (flags & STEP_REORIGIN) != 0, (flags & MG_STEP_PHYSICS) == 0);
    const bool remodel = (flags & (MG_STEP_REMODEL | MG_STEP_BOND_CHANGES)) != 0;
    const bool heal_list = heal_from_density(h, flags);
    if (flags & MG_STEP_SURROGATE) {
        enqueue_surrogate_morphogen(h, (flags & MG_STEP_PHYSICS) != 0, prof, heal_list);
    } else {
        int dflags = ((flags & MG_STEP_PHYSICS) ? 1 : 0) | ((flags & MG_STEP_GENES) ? 6 : 0);
        if (dflags) enqueue_dens(h, dflags, prof, heal_list);
    }
    bool early = false;  // FCONC is final once the morphogen stage has run
    if (io)
        for (uint32_t k = 0; k < io->nout; k++)
            if (io->out[k].buf_id == MG_FCONC) {
                if (!early) {
                    cudaEventRecord(ev[3], st);
                    cudaStreamWaitEvent(A, ev[3], 0);
                    early = true;
                }
                cudaMemcpyAsync(io->out[k].host, direct_buffer(h, MG_FCONC, false), io->out[k].bytes,
                                cudaMemcpyDeviceToHost, A);
            }
    if (early) cudaEventRecord(ev[4], A);
    flush_motion(h, prof);
    // without remodelling the integration follows the force pass and adds the incoming-bond
    // reactions itself (one kernel fewer)
    const bool in_advance = !remodel;
    if (flags & MG_STEP_PHYSICS) {
        { Mark m(h, prof, "force");
          launch_force(h->P, h->set[h->cur], h->s, h->flist_valid, h->stream, in_advance); }
    }
    if (remodel) {  // Run2Remodelling, after the gene action and before AdvanceCL
        Mark m(h, prof, "remodel");
        if (flags & MG_STEP_PHYSICS) launch_apply_breaks(h->P, h->set[h->cur], h->s, h->stream);
        const bool changes = (flags & MG_STEP_BOND_CHANGES) != 0;
        if (changes) launch_bond_changes(h->P, h->dG, h->set[h->cur], h->cold, h->s, 1.0f, h->stream);
        launch_remodel(h->P, h->dG, h->set[h->cur], h->cold, h->s, changes, !h->drifted,
                       heal_list ? h->hmem : nullptr, heal_list ? h->hmem + h->cap : nullptr, h->stream);
        h->changes_valid = changes;
    }
    if (flags & MG_STEP_PHYSICS) {
        { Mark m(h, prof, "advance");
          launch_advance(h->P, h->set[h->cur], h->s, !remodel, h->stream, (flags & MG_STEP_SPECIAL) != 0,
                         in_advance); }
        h->flist_valid = false;
    }
    if (io) {
        for (uint32_t k = 0; k < io->nout; k++)
            if (io->out[k].buf_id != MG_FCONC)
                cudaMemcpyAsync(io->out[k].host, direct_buffer(h, io->out[k].buf_id, false), io->out[k].bytes,
                                cudaMemcpyDeviceToHost, st);
        if (early) cudaStreamWaitEvent(st, ev[4], 0);
    }
}

int kernels_per_step(const mg_system* h, uint32_t flags) {
    int n = 7;  // clear, insert, scan, place, cellsort, cellsort_big, gather
    // density pass (+ its overflow pass with the fine-cell search)
    if (flags & (MG_STEP_PHYSICS | MG_STEP_GENES | MG_STEP_SURROGATE)) n += h->search == 2 ? 2 : 1;
    if (flags & MG_STEP_SURROGATE) n += 1;
    const bool remodel = (flags & (MG_STEP_REMODEL | MG_STEP_BOND_CHANGES)) != 0;
    // force (two kernels, the second folded into the integration without remodelling), advance
    if (flags & MG_STEP_PHYSICS) n += remodel ? 3 : 2;
    if (flags & (MG_STEP_REMODEL | MG_STEP_BOND_CHANGES)) n += (flags & MG_STEP_PHYSICS) ? 4 : 3;
    if (flags & MG_STEP_BOND_CHANGES) n += 1;
    return n;
}

mg_status get_graph(mg_system* h, uint32_t flags, cudaGraphExec_t* out) {
    uint64_t key = ((uint64_t)flags << 8) | ((uint64_t)h->osp << 2) | ((uint64_t)h->cur << 1) |
                   (uint64_t)h->conc_cur;
    auto it = h->graphs.find(key);
    int cur0 = h->cur, conc0 = h->conc_cur;
    if (it != h->graphs.end()) {
        *out = it->second;
        // advance the buffer state exactly as enqueue_step would
        h->cur = 1 - cur0;
        h->conc_cur = 1 - conc0;
        if (flags & (MG_STEP_GENES | MG_STEP_SURROGATE)) h->conc_cur = conc0;
        if (flags & STEP_REORIGIN) swap_ospace(h);
        return MG_OK;
    }
    DevParams saved = h->P;
    if (flags & MG_STEP_FREEZE) h->P.freeze = 1;
    cudaGraph_t g = nullptr;
    prepare_step(h, flags);
    const int osp0 = h->osp;
    // a step that is not launched leaves the buffer state where it was
    auto unwind = [&]() {
        h->cur = cur0;
        h->conc_cur = conc0;
        if (h->osp != osp0) swap_ospace(h);
    };
    MG_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step(h, flags, false);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    h->P = saved;
    if (e != cudaSuccess) {
        unwind();
        return cuda_fail(h, e, "cudaStreamEndCapture");
    }
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        unwind();
        return cuda_fail(h, e, "cudaGraphInstantiate");
    }
    h->graphs[key] = ge;
    *out = ge;
    return MG_OK;
}

void advance_state(mg_system* h, uint32_t flags);

// Whether a host buffer is page-locked (only those copies are captured into graphs).
bool host_pinned(const void* ptr) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Graph of one step with its host exchange folded in (cached by flags, buffer state and the
// exchange list: host addresses are part of the captured copies).
mg_status get_io_graph(mg_system* h, uint32_t flags, const IoPlan& io, cudaGraphExec_t* out) {
    std::string key = std::to_string(flags) + "/" + std::to_string(h->cur) + "/" + std::to_string(h->conc_cur) +
                      "/" + std::to_string(h->osp);
    char buf[96];
    for (uint32_t k = 0; k < io.nin; k++) {
        std::snprintf(buf, sizeof buf, "/i%d:%p:%zu", io.in[k].buf_id, io.in[k].host, io.in[k].bytes);
        key += buf;
    }
    for (uint32_t k = 0; k < io.nout; k++) {
        std::snprintf(buf, sizeof buf, "/o%d:%p:%zu", io.out[k].buf_id, io.out[k].host, io.out[k].bytes);
        key += buf;
    }
    const int cur0 = h->cur, conc0 = h->conc_cur;
    auto it = h->io_graphs.find(key);
    if (it != h->io_graphs.end()) {
        *out = it->second;
        advance_state(h, flags);
        return MG_OK;
    }
    for (auto& x : h->io_st)
        if (!x) MG_CUDA(h, cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
    for (auto& x : h->io_ev)
        if (!x) MG_CUDA(h, cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    DevParams saved = h->P;
    if (flags & MG_STEP_FREEZE) h->P.freeze = 1;
    cudaGraph_t g = nullptr;
    prepare_step(h, flags);
    MG_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step(h, flags, false, &io);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    h->P = saved;
    if (e != cudaSuccess) {
        h->cur = cur0;
        h->conc_cur = conc0;
        return cuda_fail(h, e, "cudaStreamEndCapture (exchange step)");
    }
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        h->cur = cur0;
        h->conc_cur = conc0;
        return cuda_fail(h, e, "cudaGraphInstantiate (exchange step)");
    }
    h->io_graphs[key] = ge;
    *out = ge;
    return MG_OK;
}

// The buffer-state change one step makes (what enqueue_step does to cur / conc_cur).
void advance_state(mg_system* h, uint32_t flags) {
    const int conc0 = h->conc_cur;
    h->cur = 1 - h->cur;
    h->conc_cur = 1 - conc0;
    if (flags & (MG_STEP_GENES | MG_STEP_SURROGATE)) h->conc_cur = conc0;
}

// The inverse of advance_state (a step whose graph was not launched).
void undo_state(mg_system* h, uint32_t flags) {
    h->cur = 1 - h->cur;
    if (!(flags & (MG_STEP_GENES | MG_STEP_SURROGATE))) h->conc_cur = 1 - h->conc_cur;
}

// Bookkeeping of a handle after nsteps graph steps (the same as run_steps does).
void after_steps(mg_system* h, uint32_t nsteps, uint32_t flags) {
    h->launches += (uint64_t)kernels_per_step(h, flags) * nsteps;
    if (flags & MG_STEP_PHYSICS)
        for (uint32_t s = 0; s < nsteps; s++) h->time = h->time + h->P.dt;
    h->phase = PHASE_SORTED;
    h->ever_sorted = true;
    h->brk_pending = false;
    h->flist_valid = (flags & MG_STEP_PHYSICS) ? false
                     : (h->search && (flags & (MG_STEP_GENES | MG_STEP_SURROGATE)));
    h->changes_valid = (flags & MG_STEP_BOND_CHANGES) != 0;
    h->drifted = (flags & MG_STEP_PHYSICS) != 0;
}

// Packed instances step physics and the plain morphogen stage (the batched sweep); the
// surrogate, remodelling and special particles run on single systems.
mg_status packed_flags_ok(mg_system* h, uint32_t flags) {
    if (h->n_inst && (flags & (MG_STEP_SURROGATE | MG_STEP_REMODEL | MG_STEP_BOND_CHANGES | MG_STEP_SPECIAL)))
        return fail(h, MG_ERR_UNSUPPORTED,
                    "packed instances step physics and the plain morphogen stage only (no surrogate, "
                    "remodelling or special particles)");
    return MG_OK;
}

mg_status run_steps(mg_system* h, uint32_t nsteps, uint32_t flags) {
    if (mg_status st0 = packed_flags_ok(h, flags)) return st0;
    if ((flags & MG_STEP_SURROGATE) && !h->sur)
        return fail(h, MG_ERR_INVALID_ARG, "surrogate step without an attached network (mg_set_surrogate)");
    if ((flags & MG_STEP_SURROGATE) && h->P.full_epi)
        return fail(h, MG_ERR_UNSUPPORTED,
                    "the surrogate step needs gene states 0 / INT_MAX without activation lists "
                    "(the network replaces the reaction and would skip the epigenetic countdowns)");
    for (uint32_t s = 0; s < nsteps; s++) {
        const bool reo = h->reorigin_period && (h->reorigin_due || h->since_reorigin + 1 >= h->reorigin_period);
        const uint32_t fs = flags | (reo ? STEP_REORIGIN : 0u);
        if (h->profile) {
            DevParams saved = h->P;
            if (flags & MG_STEP_FREEZE) h->P.freeze = 1;
            prepare_step(h, flags);
            enqueue_step(h, fs, true);
            h->P = saved;
        } else {
            cudaGraphExec_t ge = nullptr;
            mg_status st = get_graph(h, fs, &ge);
            if (st != MG_OK) return st;
            MG_CUDA(h, cudaGraphLaunch(ge, h->stream));
        }
        h->since_reorigin = reo ? 0u : h->since_reorigin + 1;
        if (reo) h->reorigin_due = false;
        h->launches += (uint64_t)kernels_per_step(h, flags);
        if (flags & MG_STEP_PHYSICS) h->time = h->time + h->P.dt;
    }
    h->phase = PHASE_SORTED;
    h->ever_sorted = true;
    h->brk_pending = false;
    h->flist_valid = (flags & MG_STEP_PHYSICS) ? false
                     : (h->search && (flags & (MG_STEP_GENES | MG_STEP_SURROGATE)));
    h->changes_valid = (flags & MG_STEP_BOND_CHANGES) != 0;
    h->drifted = (flags & MG_STEP_PHYSICS) != 0;
    if (h->profile) prof_collect(h);
    return MG_OK;
}

size_t buf_bytes(const mg_system* h, int32_t id) {
    size_t n = h->cap, C = (size_t)h->P.cells;
    switch (id) {
    case MG_FPOS: case MG_FVEL: case MG_FVEVAL: case MG_FFORCE: return 16 * n;
    case MG_FPRESS: case MG_FDENSITY: case MG_FAGE: case MG_FCOLOR: case MG_FGCELL: case MG_FGNDX:
    case MG_FBIN: case MG_FPARTICLE_ID: case MG_FMASS_RADIUS: case MG_FNERVEIDX: return 4 * n;
    case MG_FELASTIDX: return 4 * n * MG_BOND_DATA;
    case MG_FPARTICLEIDX: return 4 * n * 2 * NB;
    case MG_FCONC: return 4 * n * NTF;
    case MG_FEPIGEN: return 4 * n * NG;
    case MG_FBIN_COUNT: case MG_FBIN_OFFSET: return 4 * C;
    case MG_FBIN_COUNT_ACTIVE_GENES: case MG_FBIN_OFFSET_ACTIVE_GENES: return 4 * C * NG;
    case MG_FDENSE_LIST_LENGTHS: return 4 * NG;
    case MG_FDENSE_LISTS: return 4 * n * NG;
    case MG_FBIN_COUNT_CHANGES: case MG_FBIN_OFFSET_CHANGES: return 4 * C * MG_NUM_CHANGES;
    case MG_FDENSE_LIST_LENGTHS_CHANGES: return 4 * MG_NUM_CHANGES;
    case MG_FDENSE_LISTS_CHANGES: return 8 * n * MG_NUM_CHANGES;
    default: return 0;
    }
}

mg_status ensure_staging(mg_system* h, size_t bytes) {
    if (h->staging_bytes >= bytes) return MG_OK;
    if (h->staging) cudaFree(h->staging);
    h->staging = nullptr;
    h->staging_bytes = 0;
    cudaError_t e = cudaMalloc(&h->staging, bytes);
    if (e != cudaSuccess) return fail(h, MG_ERR_OOM, "staging buffer allocation failed");
    h->staging_bytes = bytes;
    return MG_OK;
}

uint32_t* cold_field(mg_system* h, int32_t id) {
    switch (id) {
    case MG_FAGE: return h->cold.age;
    case MG_FCOLOR: return h->cold.color;
    case MG_FPARTICLE_ID: return h->cold.pid;
    case MG_FMASS_RADIUS: return h->cold.mass_radius;
    case MG_FNERVEIDX: return h->cold.nerve;
    default: return nullptr;
    }
}

// Per-gene cell counts, offsets, dense lists and lengths from the sorted gene bits.
mg_status build_dense_lists(mg_system* h) {
    size_t C = h->P.cells, n = h->cap;
    if (!h->dense) {
        cudaError_t e = cudaMalloc(&h->dense, 4 * (2 * C * NG + n * NG + NG));
        if (e != cudaSuccess) return fail(h, MG_ERR_OOM, "dense-list buffers");
    }
    uint32_t* gcount = h->dense;
    uint32_t* goffset = gcount + C * NG;
    uint32_t* lists = goffset + C * NG;
    uint32_t* lens = lists + n * NG;
    cudaStream_t st = h->stream;
    MG_CUDA(h, cudaMemsetAsync(gcount, 0, 4 * C * NG, st));
    launch_gene_cell_counts(h->P, h->set[h->cur], h->s, gcount, st);
    for (int g = 0; g < NG; g++) {
        MG_CUDA(h, cudaMemsetAsync(h->s.scan_status, 0, sizeof(unsigned long long) * scan_status_words((uint32_t)C), st));
        MG_CUDA(h, cudaMemsetAsync(h->s.counters, 0, 4, st));
        launch_scan(gcount + g * C, goffset + g * C, (uint32_t)C, h->s.scan_status, h->s.counters,
                    nullptr, h->s.counters + 2, st);
    }
    launch_fill_u32(lists, UNDEF, n * NG, st);
    launch_gene_lists(h->P, h->set[h->cur], h->s, goffset, lists, st);
    mg_status s2 = check_device(h);
    if (s2 != MG_OK) return s2;
    // tally_denselist_lengths: len = cnt[last] + off[last] (cuda:185-194)
    std::vector<uint32_t> hl(NG);
    for (int g = 0; g < NG; g++) {
        uint32_t a = 0, b = 0;
        MG_CUDA(h, cudaMemcpy(&a, gcount + g * C + C - 1, 4, cudaMemcpyDeviceToHost));
        MG_CUDA(h, cudaMemcpy(&b, goffset + g * C + C - 1, 4, cudaMemcpyDeviceToHost));
        hl[g] = a + b;
    }
    MG_CUDA(h, cudaMemcpy(lens, hl.data(), 4 * NG, cudaMemcpyHostToDevice));
    return MG_OK;
}

// countingSortChanges (cuda:406-618) + PrefixSumChangesCL from the bonds' change words.
mg_status build_change_lists(mg_system* h) {
    const size_t C = h->P.cells, n = h->cap, K = MG_NUM_CHANGES;
    if (!h->changes) {
        cudaError_t e = cudaMalloc(&h->changes, 4 * (2 * C * K + 2 * n * K + K));
        if (e != cudaSuccess) {
            cudaGetLastError();
            h->changes = nullptr;
            return fail(h, MG_ERR_OOM, "change-list buffers");
        }
    }
    uint32_t* ccount = h->changes;
    uint32_t* coffset = ccount + C * K;
    uint32_t* lists = coffset + C * K;
    uint32_t* lens = lists + 2 * n * K;
    cudaStream_t st = h->stream;
    MG_CUDA(h, cudaMemsetAsync(ccount, 0, 4 * C * K, st));
    launch_change_cell_counts(h->P, h->set[h->cur], h->cold, h->s, ccount, st);
    for (size_t k = 0; k < K; k++) {
        MG_CUDA(h, cudaMemsetAsync(h->s.scan_status, 0, sizeof(unsigned long long) * scan_status_words((uint32_t)C), st));
        MG_CUDA(h, cudaMemsetAsync(h->s.counters, 0, 4, st));
        launch_scan(ccount + k * C, coffset + k * C, (uint32_t)C, h->s.scan_status, h->s.counters,
                    nullptr, h->s.counters + 2, st);
    }
    launch_fill_u32(lists, UNDEF, 2 * n * K, st);
    launch_change_lists(h->P, h->set[h->cur], h->cold, h->s, coffset, lists, st);
    mg_status s2 = check_device(h);
    if (s2 != MG_OK) return s2;
    std::vector<uint32_t> hl(K);
    for (size_t k = 0; k < K; k++) {
        uint32_t a = 0, b = 0;
        MG_CUDA(h, cudaMemcpy(&a, ccount + k * C + C - 1, 4, cudaMemcpyDeviceToHost));
        MG_CUDA(h, cudaMemcpy(&b, coffset + k * C + C - 1, 4, cudaMemcpyDeviceToHost));
        hl[k] = a + b;
    }
    MG_CUDA(h, cudaMemcpy(lens, hl.data(), 4 * K, cudaMemcpyHostToDevice));
    return MG_OK;
}

}  // namespace

// =============================================================================================
extern "C" {

const char* mg_version(void) { return "morphogenesis-gb300 0.1 (sm_103a)"; }

const char* mg_last_error(mg_handle h) {
    if (h) return h->err.c_str();
    return g_thread_error.c_str();
}

mg_status mg_setup_grid(mg_fparams* p, const float vol_min[3], const float vol_max[3],
                        float cell_size, int32_t gsrch_override) {
    if (!p || !vol_min || !vol_max || !(cell_size > 0.f) || !(p->psimscale > 0.f))
        return fail(nullptr, MG_ERR_INVALID_ARG, "mg_setup_grid: bad arguments");
    // SetupGrid (fluid_system.cpp:2073-2131)
    float ss = p->psimscale;
    float world_cellsize = cell_size / ss;
    long long total = 1;
    for (int k = 0; k < 3; k++) {
        p->grid_min[k] = vol_min[k];
        p->grid_max[k] = vol_max[k];
        float size = vol_max[k] - vol_min[k];
        int res = (int)ceil(size / world_cellsize);
        if (res < 1) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_setup_grid: empty volume");
        p->grid_res[k] = res;
        p->grid_size[k] = res * cell_size / ss;
        p->grid_delta[k] = (float)res / p->grid_size[k];
        total *= res;
    }
    if (total > 0x7fffffffLL) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_setup_grid: grid too large");
    p->grid_total = (int32_t)total;
    int srch = (int)(floor(2.0f * (p->psmoothradius / ss) / world_cellsize) + 1.0f);
    if (srch < 2) srch = 2;
    if (gsrch_override > 0) srch = gsrch_override;
    p->grid_srch = srch;
    return MG_OK;
}

// A system of max_points particles; n_inst > 0 adds the tables of packed instances (their
// frames, genomes and the per-particle instance ids), which mg_create_packed fills.
static mg_status create_system(const mg_fparams* params, const mg_genome* genome, uint32_t max_points,
                               uint32_t n_inst, mg_handle* out) {
    if (!out) return fail(nullptr, MG_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    mg_status st = check_params(nullptr, params);
    if (st != MG_OK) return st;
    if (!genome) return fail(nullptr, MG_ERR_INVALID_ARG, "genome is NULL");
    if (max_points == 0 || max_points >= 0x80000000u)
        return fail(nullptr, MG_ERR_INVALID_ARG, "max_points must be in [1, 2^31)");
    mg_system* h = new mg_system();
    h->params = *params;
    h->genome = *genome;
    h->cap = max_points;
    h->time = params->time;
    derive(h->P, *params, max_points);
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { delete h; return cuda_fail(nullptr, e, "cudaGetDevice"); }
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    if (h->num_sms <= 0) h->num_sms = 1;
    e = physics_init();
    if (e == cudaSuccess) e = mg::mlp_init_attributes();
    if (e != cudaSuccess) { delete h; return cuda_fail(nullptr, e, "kernel attributes"); }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete h; return cuda_fail(nullptr, e, "cudaStreamCreate"); }

    // ---- one arena for everything the step touches ----
    const size_t n = max_points, C = (size_t)params->grid_total;
    const size_t tiles = scan_status_words((uint32_t)C);
    std::vector<std::pair<void**, size_t>> plan;
    for (int k = 0; k < 2; k++) {
        Carried& c = h->set[k];
        plan.push_back({(void**)&c.pos, 16 * n});
        plan.push_back({(void**)&c.vel, 16 * n});
        plan.push_back({(void**)&c.veval, 16 * n});
        plan.push_back({(void**)&c.pidx, 48 * n});
        plan.push_back({(void**)&c.press, 4 * n});
        plan.push_back({(void**)&c.invdens, 4 * n});
        plan.push_back({(void**)&c.conc, 64 * n});
        plan.push_back({(void**)&c.genes, 4 * n});
        plan.push_back({(void**)&c.origin, 4 * n});
        if (n_inst) plan.push_back({(void**)&c.iid, 4 * n});
    }
    if (n_inst) {
        plan.push_back({(void**)&h->d_inst, sizeof(InstParams) * (size_t)n_inst});
        plan.push_back({(void**)&h->d_genomes, sizeof(DevGenome) * (size_t)n_inst});
    }
    // the two origin spaces (cold fields and bond records; the carried sets share the current)
    for (Cold* c : {&h->cold, &h->cold_alt}) {
        plan.push_back({(void**)&c->bond, 32 * NB * n});
        plan.push_back({(void**)&c->partner, 4 * NB * n});
        plan.push_back({(void**)&c->age, 4 * n});
        plan.push_back({(void**)&c->color, 4 * n});
        plan.push_back({(void**)&c->pid, 4 * n});
        plan.push_back({(void**)&c->mass_radius, 4 * n});
        plan.push_back({(void**)&c->nerve, 4 * n});
        plan.push_back({(void**)&c->change, 4 * NB * n});
    }
    plan.push_back({(void**)&h->s.cell, 4 * n});
    plan.push_back({(void**)&h->s.arank, 4 * n});
    plan.push_back({(void**)&h->s.order, 4 * n});
    plan.push_back({(void**)&h->s.okey, 8 * n});
    plan.push_back({(void**)&h->s.sorted, 4 * n});
    plan.push_back({(void**)&h->s.work, 4 * n});
    plan.push_back({(void**)&h->s.sub, n});
    plan.push_back({(void**)&h->s.subcnt, 8 * C});
    plan.push_back({(void**)&h->s.ovf, 4 * n});
    plan.push_back({(void**)&h->s.freemask, n});
    plan.push_back({(void**)&h->s.prop_cnt, 4 * n});
    plan.push_back({(void**)&h->s.prop_list, 4 * n * PROP_K});
    plan.push_back({(void**)&h->s.prop, 4 * n});
    plan.push_back({(void**)&h->s.propd, 4 * n});
    plan.push_back({(void**)&h->s.newidx, 4 * n});
    plan.push_back({(void**)&h->s.scell, 4 * n});
    plan.push_back({(void**)&h->s.force, 16 * n});
    plan.push_back({(void**)&h->s.bterm, 16 * (size_t)NB * n});
    plan.push_back({(void**)&h->s.brk, 4 * n});
    plan.push_back({(void**)&h->s.flist, 4 * (size_t)FL_CAP * n});
    plan.push_back({(void**)&h->s.fcount, 4 * n});
    plan.push_back({(void**)&h->s.count, 4 * C});
    plan.push_back({(void**)&h->s.offset, 4 * C});
    plan.push_back({(void**)&h->s.scan_status, 8 * (tiles + 1)});
    plan.push_back({(void**)&h->s.counters, 64});
    plan.push_back({(void**)&h->s.big_list, 4 * (size_t)BIG_LIST_CAP});
    plan.push_back({(void**)&h->dG, sizeof(DevGenome)});
    size_t total = 0;
    for (auto& pr : plan) total += align_up(pr.second);
    e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) {
        cudaStreamDestroy(h->stream);
        delete h;
        return fail(nullptr, MG_ERR_OOM, "device arena allocation failed (" + std::to_string(total) + " bytes)");
    }
    h->arena_bytes = total;
    char* base = (char*)h->arena;
    for (auto& pr : plan) {
        *pr.first = base;
        base += align_up(pr.second);
    }
    for (Carried& c : h->set) {
        c.bond = h->cold.bond;
        c.partner = h->cold.partner;
    }
    h->P.err = h->s.counters + 2;
    cudaMemsetAsync(h->arena, 0, total, h->stream);
    launch_init_set(max_points, h->set[0], h->stream);
    launch_init_set(max_points, h->set[1], h->stream);
    uint32_t init_counters[16] = {0};
    init_counters[3] = max_points;  // every slot counts as active until the first sort
    std::memcpy(&init_counters[7], &params->time, 4);  // device time, both parity slots
    std::memcpy(&init_counters[8], &params->time, 4);
    cudaMemcpyAsync(h->s.counters, init_counters, sizeof(init_counters), cudaMemcpyHostToDevice, h->stream);
    launch_fill_u32(h->s.cell, UNDEF, n, h->stream);
    launch_fill_u32(h->s.newidx, UNDEF, n, h->stream);
    launch_fill_u32(h->s.scell, UNDEF, n, h->stream);
    st = upload_genome(h);
    if (st == MG_OK) st = check_device(h);
    if (st != MG_OK) {
        std::string m = h->err;
        mg_destroy(h);
        return fail(nullptr, st, m);
    }
    *out = h;
    return MG_OK;
}

mg_status mg_create(const mg_fparams* params, const mg_genome* genome, uint32_t max_points,
                    mg_handle* out) {
    return create_system(params, genome, max_points, 0, out);
}

// ---- packed instances --------------------------------------------------------------------------
mg_status mg_create_packed(const mg_fparams* params, const mg_genome* genomes,
                           const uint32_t* max_points, uint32_t n_inst, mg_handle* out) {
    if (!out || !params || !genomes || !max_points || n_inst == 0)
        return fail(nullptr, MG_ERR_INVALID_ARG, "mg_create_packed: bad arguments");
    *out = nullptr;
    const mg_fparams& a = params[0];
    uint64_t cap = 0;
    long long rx = 0, ry = 0, rz = 0;
    for (uint32_t k = 0; k < n_inst; k++) {
        const mg_fparams& q = params[k];
        mg_status st = check_params(nullptr, &q);
        if (st != MG_OK) return st;
        if (max_points[k] == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_create_packed: an instance has no particles");
        cap += max_points[k];
        // everything but the stiffness, the box and the grid's placement and size is shared
        const bool same = q.psimscale == a.psimscale && q.psmoothradius == a.psmoothradius &&
            q.pradius == a.pradius && q.pmass == a.pmass && q.prest_dens == a.prest_dens &&
            q.pextstiff == a.pextstiff && q.pvisc == a.pvisc && q.psurface_t == a.psurface_t &&
            q.pdamp == a.pdamp && q.pforce_min == a.pforce_min && q.pforce_max == a.pforce_max &&
            q.pforce_freq == a.pforce_freq && q.pground_slope == a.pground_slope &&
            q.pgravity[0] == a.pgravity[0] && q.pgravity[1] == a.pgravity[1] && q.pgravity[2] == a.pgravity[2] &&
            q.paccel_limit == a.paccel_limit && q.pvel_limit == a.pvel_limit &&
            q.actuation_factor == a.actuation_factor && q.actuation_period == a.actuation_period &&
            q.grid_delta[0] == a.grid_delta[0] && q.grid_delta[1] == a.grid_delta[1] &&
            q.grid_delta[2] == a.grid_delta[2] && q.grid_srch == 3 && q.dt == a.dt &&
            q.time == a.time && q.freeze == a.freeze;
        if (!same)
            return fail(nullptr, MG_ERR_INVALID_ARG,
                        "mg_create_packed: instance " + std::to_string(k) +
                            " differs from instance 0 in more than its stiffness, box and grid "
                            "(27-cell window and equal cell size required)");
        rx = std::max<long long>(rx, q.grid_res[0]);
        rz = std::max<long long>(rz, q.grid_res[2]);
        ry += q.grid_res[1];
    }
    if (cap >= 0x80000000ull) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_create_packed: more than 2^31 particles");
    if (rx * ry * rz > 0x7fffffffLL) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_create_packed: shared grid above 2^31 cells");
    // the shared grid: instance slabs stacked along y, x and z as wide as the widest instance
    mg_fparams g = a;
    g.grid_res[0] = (int32_t)rx;
    g.grid_res[1] = (int32_t)ry;
    g.grid_res[2] = (int32_t)rz;
    g.grid_total = (int32_t)(rx * ry * rz);
    for (int d = 0; d < 3; d++) {
        g.grid_size[d] = (float)g.grid_res[d] / a.grid_delta[d];
        g.grid_max[d] = g.grid_min[d] + g.grid_size[d];
    }
    mg_handle h = nullptr;
    mg_status st = create_system(&g, &genomes[0], (uint32_t)cap, n_inst, &h);
    if (st != MG_OK) return st;
    h->n_inst = n_inst;
    h->inst.resize(n_inst);
    h->inst_count.assign(max_points, max_points + n_inst);
    std::vector<DevGenome> dg(n_inst);
    int ybase = 0;
    for (uint32_t k = 0; k < n_inst; k++) {
        const mg_fparams& q = params[k];
        InstParams& I = h->inst[k];
        std::memset(&I, 0, sizeof(I));
        for (int d = 0; d < 3; d++) {
            I.gmin[d] = q.grid_min[d];
            I.gdelta[d] = q.grid_delta[d];
            I.gcell[d] = 1.f / q.grid_delta[d];
            I.res[d] = q.grid_res[d];
            I.scanmax[d] = q.grid_res[d] - q.grid_srch;
            I.bmin[d] = q.pboundmin[d];
            I.bmax[d] = q.pboundmax[d];
        }
        I.ybase = ybase;
        I.frame_y = (float)((double)q.grid_min[1] - (double)ybase / (double)q.grid_delta[1]);
        I.istiff = q.pintstiff;
        ybase += q.grid_res[1];
        const std::string why = make_dev_genome(genomes[k], dg[k]);
        if (!why.empty() || has_activations(dg[k])) {
            mg_destroy(h);
            return fail(nullptr, MG_ERR_INVALID_ARG,
                        "mg_create_packed: genome " + std::to_string(k) + ": " +
                            (why.empty() ? std::string("activation lists are not supported") : why));
        }
    }
    // the instance of every slot, in upload order (instance 0's particles first)
    std::vector<uint32_t> iid((size_t)cap);
    size_t o = 0;
    for (uint32_t k = 0; k < n_inst; k++)
        for (uint32_t j = 0; j < max_points[k]; j++) iid[o++] = k;
    cudaStream_t s0 = h->stream;
    cudaError_t e = cudaMemcpyAsync(h->d_inst, h->inst.data(), sizeof(InstParams) * n_inst, cudaMemcpyHostToDevice, s0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_genomes, dg.data(), sizeof(DevGenome) * n_inst, cudaMemcpyHostToDevice, s0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->set[h->cur].iid, iid.data(), 4 * cap, cudaMemcpyHostToDevice, s0);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->set[1 - h->cur].iid, 0xFF, 4 * cap, s0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s0);
    if (e != cudaSuccess) {
        mg_destroy(h);
        return cuda_fail(nullptr, e, "mg_create_packed");
    }
    h->P.inst = h->d_inst;
    h->P.genomes = h->d_genomes;
    h->P.n_inst = (int)n_inst;
    clear_graphs(h);
    *out = h;
    return MG_OK;
}

mg_status mg_instance_ranges(mg_handle h, uint32_t* first, uint32_t* count) {
    if (!h || !first || !count) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    if (!h->n_inst) return fail(h, MG_ERR_INVALID_ARG, "mg_instance_ranges: not a packed system");
    if (!h->ever_sorted) return fail(h, MG_ERR_INVALID_ARG, "mg_instance_ranges: the particles have not been sorted");
    mg_status st = MG_OK;
    const uint32_t nact = read_word(h, h->s.counters + 3, &st);
    for (uint32_t k = 0; k < h->n_inst && st == MG_OK; k++) {
        const size_t cell0 = (size_t)h->inst[k].ybase * (size_t)h->P.res[2] * (size_t)h->P.res[0];
        first[k] = read_word(h, h->s.offset + cell0, &st);
    }
    for (uint32_t k = 0; k < h->n_inst; k++) count[k] = (k + 1 < h->n_inst ? first[k + 1] : nact) - first[k];
    return st;
}

mg_status mg_destroy(mg_handle h) {
    if (!h) return MG_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    clear_graphs(h);
    for (auto& m : h->marks) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
    for (cudaStream_t x : h->io_st) if (x) cudaStreamDestroy(x);
    for (cudaEvent_t x : h->io_ev) if (x) cudaEventDestroy(x);
    if (h->staging) cudaFree(h->staging);
    if (h->dense) cudaFree(h->dense);
    if (h->changes) cudaFree(h->changes);
    if (h->hmem) cudaFree(h->hmem);
    if (h->epi_mem) cudaFree(h->epi_mem);
    if (h->feat) cudaFree(h->feat);
    if (h->feat_scale) cudaFree(h->feat_scale);
    if (h->conc_plain) cudaFree(h->conc_plain);
    if (h->sur_stats) cudaFree(h->sur_stats);
    if (h->arena) cudaFree(h->arena);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return MG_OK;
}

mg_status mg_update_params(mg_handle h, const mg_fparams* p) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    if (h->n_inst) return fail(h, MG_ERR_UNSUPPORTED, "packed instances keep the parameters they were created with");
    mg_status st = check_params(h, p);
    if (st != MG_OK) return st;
    if (p->grid_total != h->params.grid_total)
        return fail(h, MG_ERR_INVALID_ARG, "grid size is fixed at mg_create");
    for (int k = 0; k < 3; k++)
        if (p->grid_res[k] != h->params.grid_res[k])
            return fail(h, MG_ERR_INVALID_ARG, "grid resolution is fixed at mg_create");
    h->params = *p;
    h->time = p->time;
    // state derive() does not compute: genome-derived flags, modes and the launch shape
    const DevParams old = h->P;
    derive(h->P, *p, h->cap);
    h->P.uniform_diff = old.uniform_diff;
    h->P.full_epi = old.full_epi;
    h->P.heal_params = old.heal_params;
    h->P.dens_warps = old.dens_warps;
    h->P.group_mode = old.group_mode;
    h->P.sub_bits = old.sub_bits;
    h->P.force_threads = old.force_threads;
    h->P.gather_threads = old.gather_threads;
    h->P.advance_threads = old.advance_threads;
    h->P.err = old.err;
    clear_graphs(h);
    // the device copy of the time (both parity slots)
    const uint32_t t2[2] = {*reinterpret_cast<const uint32_t*>(&p->time), *reinterpret_cast<const uint32_t*>(&p->time)};
    MG_CUDA(h, cudaStreamSynchronize(h->stream));
    MG_CUDA(h, cudaMemcpy(h->s.counters + 7, t2, sizeof(t2), cudaMemcpyHostToDevice));
    return MG_OK;
}

mg_status mg_update_genome(mg_handle h, const mg_genome* g) {
    if (!h || !g) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    if (h->n_inst) return fail(h, MG_ERR_UNSUPPORTED, "packed instances keep the genomes they were created with");
    mg_genome saved = h->genome;
    h->genome = *g;
    mg_status st = upload_genome(h);
    if (st != MG_OK) {
        h->genome = saved;
        upload_genome(h);
        return st;
    }
    return MG_OK;
}

mg_status mg_set_param(mg_handle h, int32_t id, float v) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    mg_fparams p = h->params;
    p.time = h->time;
    switch (id) {
    case MG_PSIMSCALE: p.psimscale = v; break;
    case MG_PVISC: p.pvisc = v; break;
    case MG_PRESTDENSITY: p.prest_dens = v; break;
    case MG_PMASS: p.pmass = v; break;
    case MG_PRADIUS: p.pradius = v; break;
    case MG_PSMOOTHRADIUS: p.psmoothradius = v; break;
    case MG_PINTSTIFF: p.pintstiff = v; break;
    case MG_PEXTSTIFF: p.pextstiff = v; break;
    case MG_PEXTDAMP: p.pdamp = v; break;
    case MG_PACCEL_LIMIT: p.paccel_limit = v; break;
    case MG_PVEL_LIMIT: p.pvel_limit = v; break;
    case MG_PGROUND_SLOPE: p.pground_slope = v; break;
    case MG_PFORCE_MIN: p.pforce_min = v; break;
    case MG_PFORCE_MAX: p.pforce_max = v; break;
    case MG_PFORCE_FREQ: p.pforce_freq = v; break;
    case MG_PSURFACE_TENSION: p.psurface_t = v; break;
    case MG_PACTUATION_FACTOR: p.actuation_factor = v; break;
    case MG_PACTUATION_PERIOD: p.actuation_period = v; break;
    case MG_PDT: p.dt = v; break;
    case MG_PTIME: p.time = v; break;
    case MG_PFREEZE: p.freeze = v != 0.f; break;
    default: return fail(h, MG_ERR_INVALID_ARG, "unknown parameter id " + std::to_string(id));
    }
    return mg_update_params(h, &p);
}

mg_status mg_get_params(mg_handle h, mg_fparams* out) {
    if (!h || !out) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    *out = h->params;
    out->time = h->time;
    return MG_OK;
}

mg_status mg_buffer_bytes(mg_handle h, int32_t id, size_t* bytes) {
    if (!h || !bytes) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    *bytes = buf_bytes(h, id);
    if (*bytes == 0) return fail(h, MG_ERR_INVALID_ARG, "buffer id not exchanged by this pipeline");
    return MG_OK;
}

static mg_status enqueue_upload(mg_handle h, int32_t id, const void* host, size_t bytes) {
    if (!h || !host) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    size_t want = buf_bytes(h, id);
    if (want == 0 || id == MG_FBIN || id == MG_FBIN_COUNT || id == MG_FBIN_OFFSET ||
        id == MG_FBIN_COUNT_ACTIVE_GENES || id == MG_FBIN_OFFSET_ACTIVE_GENES ||
        id == MG_FDENSE_LIST_LENGTHS || id == MG_FDENSE_LISTS)
        return fail(h, MG_ERR_INVALID_ARG, "buffer id " + std::to_string(id) + " cannot be uploaded");
    if (bytes != want)
        return fail(h, MG_ERR_INVALID_ARG, "buffer " + std::to_string(id) + ": expected " +
                                               std::to_string(want) + " bytes, got " + std::to_string(bytes));
    cudaStream_t st = h->stream;
    Carried& c = h->set[h->cur];
    void* dst = nullptr;
    h->flist_valid = false;
    if (id == MG_FPOS) {
        h->drifted = true;        // positions no longer those the cells were built from
        h->reorigin_due = true;   // and the upload order is no guide to the sorted order
    }
    switch (id) {
    case MG_FPOS: dst = c.pos; break;
    case MG_FVEL: dst = c.vel; break;
    case MG_FVEVAL: dst = c.veval; break;
    case MG_FFORCE: dst = h->s.force; break;
    case MG_FPRESS: dst = c.press; break;
    case MG_FDENSITY: dst = c.invdens; break;
    case MG_FPARTICLEIDX: dst = c.pidx; break;
    case MG_FCONC: dst = h->conc_species_major ? nullptr : conc_of(h, h->conc_cur); break;
    case MG_FGCELL: case MG_FGNDX: return MG_OK;  // recomputed by insert
    default: break;
    }
    if (id == MG_FEPIGEN) {
        // values other than 0 and INT_MAX are epigenetic countdowns: keep the full state
        const uint32_t* w = (const uint32_t*)host;
        bool countdown = false;
        for (size_t k = 0; k < (size_t)NG * h->cap && !countdown; k++)
            countdown = w[k] != 0u && w[k] != MG_EPIGEN_ACTIVE;
        if (countdown) {
            mg_status s2 = enable_full_epi(h);
            if (s2 != MG_OK) return s2;
        }
        if (h->P.full_epi) {
            MG_CUDA(h, cudaMemcpyAsync(c.epi, host, bytes, cudaMemcpyHostToDevice, st));
            launch_words_to_bits(h->cap, c, st);
            return MG_OK;
        }
    }
    if (dst) {
        MG_CUDA(h, cudaMemcpyAsync(dst, host, bytes, cudaMemcpyHostToDevice, st));
        return MG_OK;
    }
    mg_status s2 = ensure_staging(h, bytes);
    if (s2 != MG_OK) return s2;
    MG_CUDA(h, cudaMemcpyAsync(h->staging, host, bytes, cudaMemcpyHostToDevice, st));
    const uint32_t* sref = (const uint32_t*)h->staging;
    if (id == MG_FCONC) {  // species-major host layout
        launch_conc_transpose(h->cap, (const float*)sref, conc_of(h, h->conc_cur), false, st);
    } else if (id == MG_FELASTIDX) {
        launch_import_bonds(h->P, sref, c, h->cold, st);
        h->brk_pending = false;
    } else if (id == MG_FEPIGEN) {
        launch_import_epigen(h->P, sref, c, h->s.counters + 2, st);
    } else if (uint32_t* f = cold_field(h, id)) {
        launch_import_cold(h->P, sref, c, f, st);
    } else {
        return fail(h, MG_ERR_INVALID_ARG, "buffer id " + std::to_string(id) + " cannot be uploaded");
    }
    return MG_OK;
}

mg_status mg_upload(mg_handle h, int32_t id, const void* host, size_t bytes) {
    mg_status st = enqueue_upload(h, id, host, bytes);
    return st != MG_OK ? st : check_device(h);
}

static mg_status enqueue_download(mg_handle h, int32_t id, void* host, size_t bytes) {
    if (!h || !host) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    size_t want = buf_bytes(h, id);
    if (want == 0) return fail(h, MG_ERR_INVALID_ARG, "buffer id " + std::to_string(id) + " not exchanged");
    if (bytes != want)
        return fail(h, MG_ERR_INVALID_ARG, "buffer " + std::to_string(id) + ": expected " +
                                               std::to_string(want) + " bytes, got " + std::to_string(bytes));
    cudaStream_t st = h->stream;
    Carried& c = h->set[h->cur];
    const void* src = nullptr;
    switch (id) {
    case MG_FPOS: src = c.pos; break;
    case MG_FVEL: src = c.vel; break;
    case MG_FVEVAL: src = c.veval; break;
    case MG_FFORCE: src = h->s.force; break;
    case MG_FPRESS: src = c.press; break;
    case MG_FDENSITY: src = c.invdens; break;
    case MG_FPARTICLEIDX: src = c.pidx; break;
    case MG_FCONC: src = h->conc_species_major ? nullptr : conc_of(h, h->conc_cur); break;
    case MG_FBIN_COUNT: src = h->s.count; break;
    case MG_FBIN_OFFSET: src = h->s.offset; break;
    default: break;
    }
    if (id == MG_FEPIGEN && h->P.full_epi) src = c.epi;
    if (id == MG_FCONC && h->conc_species_major) {
        mg_status s2 = ensure_staging(h, bytes);
        if (s2 != MG_OK) return s2;
        launch_conc_transpose(h->cap, conc_of(h, h->conc_cur), (float*)h->staging, true, st);
        MG_CUDA(h, cudaMemcpyAsync(host, h->staging, bytes, cudaMemcpyDeviceToHost, st));
        return MG_OK;
    }
    if (src) {
        MG_CUDA(h, cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, st));
        return MG_OK;
    }
    if (id == MG_FBIN_COUNT_ACTIVE_GENES || id == MG_FBIN_OFFSET_ACTIVE_GENES ||
        id == MG_FDENSE_LIST_LENGTHS || id == MG_FDENSE_LISTS) {
        if (h->phase != PHASE_SORTED) return fail(h, MG_ERR_INVALID_ARG, "dense lists exist after a sort");
        mg_status s2 = build_dense_lists(h);
        if (s2 != MG_OK) return s2;
        size_t C = h->P.cells, n = h->cap;
        const uint32_t* base = h->dense;
        const uint32_t* p = id == MG_FBIN_COUNT_ACTIVE_GENES ? base
                          : id == MG_FBIN_OFFSET_ACTIVE_GENES ? base + C * NG
                          : id == MG_FDENSE_LISTS ? base + 2 * C * NG
                          : base + 2 * C * NG + n * NG;
        MG_CUDA(h, cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, st));
        return MG_OK;
    }
    if (id == MG_FBIN_COUNT_CHANGES || id == MG_FBIN_OFFSET_CHANGES ||
        id == MG_FDENSE_LIST_LENGTHS_CHANGES || id == MG_FDENSE_LISTS_CHANGES) {
        if (h->phase != PHASE_SORTED) return fail(h, MG_ERR_INVALID_ARG, "change lists exist after a sort");
        mg_status s2 = build_change_lists(h);
        if (s2 != MG_OK) return s2;
        const size_t C = h->P.cells, n = h->cap, K = MG_NUM_CHANGES;
        const uint32_t* base = h->changes;
        const uint32_t* p = id == MG_FBIN_COUNT_CHANGES ? base
                          : id == MG_FBIN_OFFSET_CHANGES ? base + C * K
                          : id == MG_FDENSE_LISTS_CHANGES ? base + 2 * C * K
                          : base + 2 * C * K + 2 * n * K;
        MG_CUDA(h, cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, st));
        return MG_OK;
    }
    mg_status s2 = ensure_staging(h, bytes);
    if (s2 != MG_OK) return s2;
    uint32_t* sref = (uint32_t*)h->staging;
    if (id == MG_FELASTIDX) {
        launch_export_bonds(h->P, c, h->cold, h->s, h->brk_pending, sref, st);
    } else if (id == MG_FEPIGEN) {
        launch_export_epigen(h->P, c, h->s, sref, st);
    } else if (uint32_t* f = cold_field(h, id)) {
        launch_export_cold(h->P, c, h->s, f, id == MG_FPARTICLE_ID ? NO_PARTNER : 0u, sref, st);
    } else if (id == MG_FGCELL || id == MG_FGNDX || id == MG_FBIN) {
        int which = id == MG_FGCELL ? 0 : id == MG_FGNDX ? 1 : 2;
        if (h->phase == PHASE_UNSORTED && !h->ever_sorted && which != 2)
            launch_fill_u32(sref, UNDEF, h->cap, st);
        else
            launch_export_grid_index(h->P, h->s, which, h->phase == PHASE_INSERTED ? 1 : 2, sref, st);
    } else {
        return fail(h, MG_ERR_INVALID_ARG, "buffer id " + std::to_string(id) + " not exchanged");
    }
    MG_CUDA(h, cudaMemcpyAsync(host, sref, bytes, cudaMemcpyDeviceToHost, st));
    return MG_OK;
}

mg_status mg_download(mg_handle h, int32_t id, void* host, size_t bytes) {
    mg_status st = enqueue_download(h, id, host, bytes);
    return st != MG_OK ? st : check_device(h);
}

// One host exchange cycle with a single synchronisation: uploads, steps, downloads, all
// enqueued in order on the handle's stream.
mg_status mg_step_io(mg_handle h, const mg_io* in, uint32_t nin, uint32_t nsteps, uint32_t flags,
                     const mg_io* out, uint32_t nout) {
    if (!h || (nin && !in) || (nout && !out)) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    Range r("mg_step_io");
    if (h->profile) return fail(h, MG_ERR_INVALID_ARG, "mg_step_io: profiling is on");
    if (mg_status st0 = packed_flags_ok(h, flags)) return st0;
    // Plain-copy buffers with the right sizes in page-locked host memory: the copies go into the
    // steps' graphs, overlapped with the first step (uploads) and the last (downloads).
    // Anything else goes the sequential way below.
    bool direct = nsteps > 0 && (flags & (MG_STEP_PHYSICS | MG_STEP_GENES | MG_STEP_SURROGATE)) != 0;
    for (uint32_t k = 0; direct && k < nin; k++)
        direct = in[k].host && direct_buffer(h, in[k].buf_id, true) &&
                 in[k].bytes == buf_bytes(h, in[k].buf_id) && host_pinned(in[k].host);
    for (uint32_t k = 0; direct && k < nout; k++)
        direct = out[k].host && direct_buffer(h, out[k].buf_id, false) &&
                 out[k].bytes == buf_bytes(h, out[k].buf_id) && host_pinned(out[k].host);
    if (direct) {
        if ((flags & MG_STEP_SURROGATE) && (!h->sur || h->P.full_epi)) return run_steps(h, nsteps, flags);
        if (nin) h->flist_valid = false;
        for (uint32_t s = 0; s < nsteps; s++) {
            IoPlan plan;
            if (s == 0) { plan.in = in; plan.nin = nin; }
            if (s + 1 == nsteps) { plan.out = out; plan.nout = nout; }
            cudaGraphExec_t ge = nullptr;
            mg_status st = (plan.nin || plan.nout) ? get_io_graph(h, flags, plan, &ge) : get_graph(h, flags, &ge);
            if (st != MG_OK) return st;
            MG_CUDA(h, cudaGraphLaunch(ge, h->stream));
        }
        after_steps(h, nsteps, flags);
        // the first step's gather in parts: the concentrations and the motion fields after
        // their uploads
        bool conc_in = false, motion_in = false;
        for (uint32_t k = 0; k < nin; k++) {
            conc_in |= in[k].buf_id == MG_FCONC;
            motion_in |= motion_buffer(in[k].buf_id);
        }
        h->launches += (conc_in ? 1 : 0) + (motion_in ? 1 : 0);
        return check_device(h);
    }
    for (uint32_t k = 0; k < nin; k++) {
        mg_status st = enqueue_upload(h, in[k].buf_id, in[k].host, in[k].bytes);
        if (st != MG_OK) return st;
    }
    if (nsteps) {
        mg_status st = run_steps(h, nsteps, flags);
        if (st != MG_OK) return st;
    }
    for (uint32_t k = 0; k < nout; k++) {
        mg_status st = enqueue_download(h, out[k].buf_id, out[k].host, out[k].bytes);
        if (st != MG_OK) return st;
    }
    return check_device(h);
}

mg_status mg_host_alloc(size_t bytes, void** out) {
    if (!out || bytes == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_host_alloc: bad arguments");
    cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaHostAlloc");
    return MG_OK;
}

mg_status mg_host_free(void* ptr) {
    if (!ptr) return MG_OK;
    cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaFreeHost");
    return MG_OK;
}

mg_status mg_get_counts(mg_handle h, uint32_t* num_points, uint32_t* active_points) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    mg_status st = check_device(h);
    if (st != MG_OK) return st;
    uint32_t n = read_word(h, h->s.counters + 3, &st);
    if (st != MG_OK) return st;
    uint32_t a = n;
    if (!h->n_inst && (h->ever_sorted || h->phase == PHASE_INSERTED)) {
        const DevParams& P = h->P;
        long long corner = ((long long)P.scanmax[1] * P.res[2] + P.scanmax[2]) * P.res[0] + P.scanmax[0];
        if (corner >= 0 && corner < (long long)P.cells) a = read_word(h, h->s.offset + corner, &st);
    }
    if (num_points) *num_points = n;
    if (active_points) *active_points = a;
    return st;
}

mg_status mg_insert_particles(mg_handle h) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    enqueue_insert_rank(h, false);
    h->phase = PHASE_INSERTED;
    return check_device(h);
}

mg_status mg_prefix_sum_cells(mg_handle h) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    if (h->phase != PHASE_INSERTED) return fail(h, MG_ERR_INVALID_ARG, "prefix sum needs mg_insert_particles first");
    cudaStream_t st = h->stream;
    cudaMemsetAsync(h->s.scan_status, 0, sizeof(unsigned long long) * scan_status_words(h->P.cells), st);
    cudaMemsetAsync(h->s.counters, 0, 4, st);
    launch_scan(h->s.count, h->s.offset, h->P.cells, h->s.scan_status, h->s.counters,
                h->s.counters + 3, h->s.counters + 2, st);
    return check_device(h);
}

mg_status mg_counting_sort_full(mg_handle h) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    if (h->phase != PHASE_INSERTED) return fail(h, MG_ERR_INVALID_ARG, "counting sort needs mg_insert_particles first");
    enqueue_gather(h, false);
    h->phase = PHASE_SORTED;
    h->ever_sorted = true;
    h->brk_pending = false;
    return check_device(h);
}

static mg_status need_sorted(mg_handle h) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    // Neighbour loops index cells through the sorted particles' cells; after an insert without
    // the sort those no longer match the counts, so the sort must come first.
    if (h->phase != PHASE_SORTED) return fail(h, MG_ERR_INVALID_ARG, "this stage needs a counting sort first");
    return MG_OK;
}

mg_status mg_compute_pressure(mg_handle h) {
    mg_status st = need_sorted(h);
    if (st != MG_OK) return st;
    enqueue_dens(h, 1, false);
    return check_device(h);
}

mg_status mg_compute_force(mg_handle h) {
    mg_status st = need_sorted(h);
    if (st != MG_OK) return st;
    launch_force(h->P, h->set[h->cur], h->s, h->flist_valid, h->stream);
    launch_apply_breaks(h->P, h->set[h->cur], h->s, h->stream);
    return check_device(h);
}

mg_status mg_compute_diffusion(mg_handle h) {
    mg_status st = need_sorted(h);
    if (st != MG_OK) return st;
    enqueue_dens(h, 2, false);
    return check_device(h);
}

mg_status mg_compute_genes(mg_handle h) {
    mg_status st = need_sorted(h);
    if (st != MG_OK) return st;
    enqueue_dens(h, 4, false);
    return check_device(h);
}

mg_status mg_advance(mg_handle h) {
    mg_status st = need_sorted(h);
    if (st != MG_OK) return st;
    launch_advance(h->P, h->set[h->cur], h->s, false, h->stream);
    h->flist_valid = false;
    h->drifted = true;
    h->time = h->time + h->P.dt;
    return check_device(h);
}

mg_status mg_run_remodelling(mg_handle h) {
    if (h && h->n_inst) return packed_flags_ok(h, MG_STEP_REMODEL);
    mg_status st = need_sorted(h);
    if (st != MG_OK) return st;
    launch_remodel(h->P, h->dG, h->set[h->cur], h->cold, h->s, h->changes_valid, !h->drifted, nullptr,
                   nullptr, h->stream);
    return check_device(h);
}

mg_status mg_compute_bond_changes(mg_handle h, uint32_t steps_per_inner_loop) {
    if (h && h->n_inst) return packed_flags_ok(h, MG_STEP_BOND_CHANGES);
    mg_status st = need_sorted(h);
    if (st != MG_OK) return st;
    if (steps_per_inner_loop == 0) return fail(h, MG_ERR_INVALID_ARG, "steps_per_InnerPhysicalLoop is 0");
    launch_bond_changes(h->P, h->dG, h->set[h->cur], h->cold, h->s, (float)steps_per_inner_loop, h->stream);
    h->changes_valid = true;
    return check_device(h);
}

mg_status mg_get_time(mg_handle h, float* time) {
    if (!h || !time) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    *time = h->time;
    return MG_OK;
}

mg_status mg_zero_vel(mg_handle h) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    const Carried& c = h->set[h->cur];
    MG_CUDA(h, cudaMemsetAsync(c.vel, 0, sizeof(float4) * h->cap, h->stream));
    MG_CUDA(h, cudaMemsetAsync(c.veval, 0, sizeof(float4) * h->cap, h->stream));
    return check_device(h);
}

mg_status mg_run_remodelling_steps(mg_handle h, uint32_t steps_per_inner_loop) {
    mg_status st = mg_compute_bond_changes(h, steps_per_inner_loop);
    if (st == MG_OK) st = mg_run_remodelling(h);
    return st;
}

mg_status mg_run_physical_sort(mg_handle h) {
    mg_status st = mg_insert_particles(h);
    if (st == MG_OK) st = mg_prefix_sum_cells(h);
    if (st == MG_OK) st = mg_counting_sort_full(h);
    return st;
}

mg_status mg_run_inner_physical_loop(mg_handle h) {
    mg_status st = mg_compute_pressure(h);
    if (st == MG_OK) st = mg_compute_force(h);
    if (st == MG_OK) st = mg_advance(h);
    return st;
}

mg_status mg_run_gene_action(mg_handle h) {
    mg_status st = mg_compute_diffusion(h);
    if (st == MG_OK) st = mg_compute_genes(h);
    return st;
}

mg_status mg_step(mg_handle h, uint32_t nsteps, uint32_t flags) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    Range r("mg_step");
    mg_status st = run_steps(h, nsteps, flags);
    if (st != MG_OK) return st;
    return check_device(h);
}

mg_status mg_synchronize(mg_handle h) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    return check_device(h);
}

mg_status mg_time_steps(mg_handle h, uint32_t nsteps, uint32_t flags, float* ms) {
    if (!h || !ms) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    cudaEvent_t a, b;
    MG_CUDA(h, cudaEventCreate(&a));
    MG_CUDA(h, cudaEventCreate(&b));
    MG_CUDA(h, cudaEventRecord(a, h->stream));
    mg_status st = run_steps(h, nsteps, flags);
    cudaEventRecord(b, h->stream);
    cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = t;
    if (st != MG_OK) return st;
    return check_device(h);
}

mg_status mg_set_option(mg_handle h, int32_t option, int32_t value) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    switch (option) {
    case MG_OPT_NEIGHBOR_SEARCH:
        if (value < 0 || value > 2) return fail(h, MG_ERR_INVALID_ARG, "neighbour search is 0, 1 or 2");
        if (h->n_inst && value != 1)
            return fail(h, MG_ERR_UNSUPPORTED, "packed instances use the warp-cooperative search (1)");
        if (value == 2 && h->P.gsrch != 3)
            return fail(h, MG_ERR_UNSUPPORTED, "the fine-cell search needs the 27-cell window (gsrch 3)");
        if (value == 2) h->P.sub_bits = 1;  // its sub-cells are the 2x2x2 halves of a cell
        // the fine-cell search reads sub-cell tables that only a sort made for it writes
        if (value == 2 && h->search != 2 && h->phase == PHASE_SORTED) h->phase = PHASE_UNSORTED;
        h->search = value;
        h->flist_valid = false;
        clear_graphs(h);
        return MG_OK;
    case MG_OPT_HEAL_PARAMS:
        if (value < 0 || value > 1) return fail(h, MG_ERR_INVALID_ARG, "heal parameters are 0 or 1");
        h->P.heal_params = value;
        clear_graphs(h);
        return MG_OK;
    case MG_OPT_CONC_LAYOUT:
        if (value < 0 || value > 1) return fail(h, MG_ERR_INVALID_ARG, "FCONC layout is 0 or 1");
        h->conc_species_major = value;
        return MG_OK;
    case MG_OPT_REORIGIN_PERIOD:
        if (value < 0) return fail(h, MG_ERR_INVALID_ARG, "re-origin period is 0 (never) or more steps");
        h->reorigin_period = (uint32_t)value;
        return MG_OK;
    default:
        return fail(h, MG_ERR_INVALID_ARG, "unknown option " + std::to_string(option));
    }
}

mg_status mg_profile_enable(mg_handle h, int32_t enable) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    h->profile = enable != 0;
    if (enable) h->prof.clear();
    return MG_OK;
}

mg_status mg_profile_read(mg_handle h, int32_t max_slots, char* names, uint32_t* launches,
                          double* total_ms, int32_t* nslots) {
    if (!h || !nslots) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    int n = (int)h->prof.size();
    *nslots = n;
    for (int k = 0; k < n && k < max_slots; k++) {
        if (names) {
            std::memset(names + 32 * k, 0, 32);
            std::strncpy(names + 32 * k, h->prof[k].name.c_str(), 31);
        }
        if (launches) launches[k] = h->prof[k].launches;
        if (total_ms) total_ms[k] = h->prof[k].ms;
    }
    return MG_OK;
}

// Compulsory DRAM bytes of each kernel (own-particle arrays read/written once; neighbour
// reads are served from cache because the particles are sorted by cell).
mg_status mg_algorithmic_bytes(mg_handle h, const char* kernel, uint32_t flags,
                               double* bpp, double* bpc) {
    if (!bpp || !bpc) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    struct K { const char* name; double per_particle, per_cell; };
    const bool phys = flags & MG_STEP_PHYSICS, genes = flags & (MG_STEP_GENES | MG_STEP_SURROGATE);
    // Frozen compulsory traffic per particle-step (each stage reads and writes its own
    // particles' arrays once; neighbour and partner data assumed cache-resident because the
    // particles are sorted), independent of this build's data layout:
    //   bin 24 (pos 16, cell 4, rank 4); scan 12 per cell (count read, offset write, count
    //   clear); sort 728 (carried state 336 read + 336 written: pos/vel/veval 48, six bonds x
    //   (partner, rest length, modulus, damping, elastic limit, two integrators) 168, incoming
    //   table 48, id 4, concentrations 64, gene word 4; own cell and rank 8; the six partners'
    //   cell and rank 48); density 24 (pos 16, pressure 4, 1/density 4); morphogen stage 148
    //   (pos 16, concentrations 64 read + 64 written, gene word 4); force 272 (pos 16, veval 16,
    //   pressure 4, 1/density 4, bond parameters 120, integrators read + written 96, force 16);
    //   integration 116 (pos/vel/veval/force 64 read, cell 4, pos/vel/veval 48 written).
    // Plain full step: 1,312 bytes per particle + 12 per cell.
    const double dens = (phys ? 24.0 : 0.0) + (genes ? 148.0 : 0.0);
    const K table[] = {
        {"insert", 24, 0},
        {"scan", 0, 12},
        {"place", 8, 0},       // own cell and rank
        {"cellsort", 0, 0},    // the stable in-cell order is this build's own work (D1 rank)
        {"gather", 720, 0},    // carried state read + written, partners' cell and rank
        {"pressure", phys ? 24.0 : 0.0, 0},
        {"density_diffusion_genes", dens, 0},
        {"diffusion_genes", genes ? 148.0 : 0.0, 0},
        {"force", phys ? 272.0 : 0.0, 0},
        {"advance", phys ? 116.0 : 0.0, 0},
    };
    if (kernel) {
        for (const K& k : table)
            if (std::strcmp(k.name, kernel) == 0) {
                *bpp = k.per_particle;
                *bpc = k.per_cell;
                return MG_OK;
            }
        return fail(h, MG_ERR_INVALID_ARG, std::string("unknown kernel ") + kernel);
    }
    double p = 0, c = 0;
    for (const K& k : table) {
        if (!std::strcmp(k.name, "pressure") || !std::strcmp(k.name, "diffusion_genes")) continue;
        if (!std::strcmp(k.name, "density_diffusion_genes")) { p += dens; continue; }
        p += k.per_particle;
        c += k.per_cell;
    }
    *bpp = p;
    *bpc = c;
    return MG_OK;
}

// ---- learned morphogen surrogate ------------------------------------------------------------
static mg_status mlp_fail(cudaError_t e, const char* where) {
    if (e == cudaErrorTimeout) {
        char msg[200];
        std::snprintf(msg, sizeof msg, "%s: a tensor-core completion wait gave up (bounded spin)", where);
        return fail(nullptr, MG_ERR_DEVICE_TIMEOUT, msg);
    }
    return cuda_fail(nullptr, e, where);
}

mg_status mg_mlp_create(uint64_t seed, mg_mlp* out) {
    if (!out) return fail(nullptr, MG_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    mg_mlp m = new mg_mlp_s();
    cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = mg::mlp_init_attributes();
    if (e == cudaSuccess) e = mg::mlp_alloc(&m->m, seed, m->st);
    if (e != cudaSuccess) {
        mg::mlp_free(&m->m);
        if (m->st) cudaStreamDestroy(m->st);
        delete m;
        return mlp_fail(e, "mg_mlp_create");
    }
    *out = m;
    return MG_OK;
}

mg_status mg_mlp_destroy(mg_mlp m) {
    if (!m) return MG_OK;
    cudaStreamSynchronize(m->st);
    mg::mlp_free(&m->m);
    cudaStreamDestroy(m->st);
    delete m;
    return MG_OK;
}

mg_status mg_mlp_sizes(size_t* param_count, size_t* norm_count) {
    if (param_count) *param_count = mg::P_COUNT;
    if (norm_count) *norm_count = mg::NORM_COUNT;
    return MG_OK;
}

mg_status mg_mlp_get_params(mg_mlp m, float* host, size_t count) {
    if (!m || !host || count != (size_t)mg::P_COUNT) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_get_params");
    cudaError_t e = mg::mlp_get_params(&m->m, host);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_mlp_get_params");
}

mg_status mg_mlp_set_params(mg_mlp m, const float* host, size_t count) {
    if (!m || !host || count != (size_t)mg::P_COUNT) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_set_params");
    cudaError_t e = mg::mlp_set_params(&m->m, host);
    if (e == cudaSuccess) e = mg::mlp_refresh_inference(&m->m);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_mlp_set_params");
}

mg_status mg_mlp_get_norm(mg_mlp m, float* host, size_t count) {
    if (!m || !host || count != (size_t)mg::NORM_COUNT) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_get_norm");
    cudaError_t e = mg::mlp_get_norm(&m->m, host);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_mlp_get_norm");
}

mg_status mg_mlp_set_norm(mg_mlp m, const float* host, size_t count) {
    if (!m || !host || count != (size_t)mg::NORM_COUNT) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_set_norm");
    cudaError_t e = mg::mlp_set_norm(&m->m, host);
    if (e == cudaSuccess) e = mg::mlp_refresh_inference(&m->m);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_mlp_set_norm");
}

mg_status mg_mlp_gradients(mg_mlp m, const float* x, const float* y, uint32_t n, float* grads,
                           double* loss) {
    if (!m || !x || !y || !grads || n == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_gradients");
    float *dx = nullptr, *dy = nullptr;
    cudaError_t e = cudaMalloc(&dx, 4ull * n * (mg::MLP_IN + mg::MLP_OUT));
    if (e != cudaSuccess) return fail(nullptr, MG_ERR_OOM, "mg_mlp_gradients: device buffers");
    dy = dx + (size_t)n * mg::MLP_IN;
    e = cudaMemcpyAsync(dx, x, 4ull * n * mg::MLP_IN, cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y, 4ull * n * mg::MLP_OUT, cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) e = mg::mlp_grad(&m->m, dx, dy, n, grads, loss);
    cudaStreamSynchronize(m->st);
    cudaFree(dx);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_mlp_gradients");
}

mg_status mg_mlp_infer(mg_mlp m, const float* x, uint32_t n, float* y) {
    if (!m || !x || !y || n == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_infer");
    std::vector<__nv_bfloat16> xb((size_t)n * mg::MLP_IN);
    for (size_t i = 0; i < xb.size(); i++) xb[i] = __float2bfloat16(x[i]);
    void* mem = nullptr;
    const size_t fb = sizeof(__nv_bfloat16) * xb.size(), cb = 4ull * n * mg::MLP_OUT;
    cudaError_t e = cudaMalloc(&mem, fb + 2 * cb + 256);
    if (e != cudaSuccess) return fail(nullptr, MG_ERR_OOM, "mg_mlp_infer: device buffers");
    char* b = (char*)mem;
    __nv_bfloat16* feat = (__nv_bfloat16*)b;
    float* cin = (float*)(b + ((fb + 255) & ~(size_t)255));
    float* cout = cin + (size_t)n * mg::MLP_OUT;
    uint32_t* err = (uint32_t*)(cout + (size_t)n * mg::MLP_OUT);
    e = cudaMemcpyAsync(feat, xb.data(), fb, cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cin, 0, cb + cb + 64, m->st);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    CUtensorMap map;
    if (e == cudaSuccess) e = mg::make_feat_map(feat, n, &map);
    if (e == cudaSuccess) {
        mg::launch_mlp_infer(&m->m, map, nullptr, cin, nullptr, cout, nullptr, nullptr, n, nullptr, 0, 0, 0.f,
                             nullptr, err, sms, m->st);
        e = cudaGetLastError();
    }
    uint32_t herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(y, cout, cb, cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
    cudaFree(mem);
    if (e != cudaSuccess) return mlp_fail(e, "mg_mlp_infer");
    if (herr) return fail(nullptr, MG_ERR_DEVICE_TIMEOUT, "mg_mlp_infer: tensor-core completion wait gave up");
    return MG_OK;
}

mg_status mg_dataset_create(uint64_t capacity, mg_dataset* out) {
    if (!out || capacity == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_dataset_create");
    mg_dataset d = new mg_dataset_s();
    cudaError_t e = cudaMalloc(&d->dx, 4ull * capacity * (mg::MLP_IN + mg::MLP_OUT));
    if (e != cudaSuccess) {
        delete d;
        return fail(nullptr, MG_ERR_OOM, "mg_dataset_create: device buffers");
    }
    d->dy = d->dx + capacity * mg::MLP_IN;
    d->capacity = capacity;
    *out = d;
    return MG_OK;
}

mg_status mg_dataset_destroy(mg_dataset d) {
    if (!d) return MG_OK;
    cudaDeviceSynchronize();
    cudaFree(d->dx);
    delete d;
    return MG_OK;
}

mg_status mg_dataset_size(mg_dataset d, uint64_t* n) {
    if (!d || !n) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_dataset_size");
    *n = d->size;
    return MG_OK;
}

mg_status mg_dataset_read(mg_dataset d, uint64_t first, uint32_t n, float* x, float* y) {
    if (!d || first + n > d->size) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_dataset_read: range");
    cudaError_t e = cudaSuccess;
    if (x) e = cudaMemcpy(x, d->dx + first * mg::MLP_IN, 4ull * n * mg::MLP_IN, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && y) e = cudaMemcpy(y, d->dy + first * mg::MLP_OUT, 4ull * n * mg::MLP_OUT, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_dataset_read");
}

mg_status mg_dataset_capture(mg_dataset d, mg_handle h, uint32_t flags) {
    if (!d || !h) return fail(h, MG_ERR_INVALID_ARG, "mg_dataset_capture: NULL argument");
    if (h->n_inst) return packed_flags_ok(h, MG_STEP_SURROGATE);
    if (d->size + h->cap > d->capacity) return fail(h, MG_ERR_LIST_OVERFLOW, "mg_dataset_capture: dataset full");
    enqueue_insert_rank(h, false);
    enqueue_gather(h, false);
    DensExtra X{};
    X.cap_x = d->dx + d->size * mg::MLP_IN;
    X.cap_y = d->dy + d->size * mg::MLP_OUT;
    const int cin = h->conc_cur, cout = 1 - h->conc_cur;
    launch_dens(h->P, h->dG, h->hG, h->set[h->cur], conc_of(h, cin), conc_of(h, cout), h->s, 1 | 2 | 4 | 16,
                h->search, h->num_sms, h->stream, &X);
    h->conc_cur = cout;
    h->flist_valid = h->search != 0;
    if (flags & MG_STEP_PHYSICS) {
        launch_force(h->P, h->set[h->cur], h->s, h->flist_valid, h->stream);
        launch_advance(h->P, h->set[h->cur], h->s, true, h->stream);
        h->flist_valid = false;
        h->drifted = true;
        h->time = h->time + h->P.dt;
    }
    h->phase = PHASE_SORTED;
    h->ever_sorted = true;
    h->brk_pending = false;
    mg_status st = check_device(h);
    if (st != MG_OK) return st;
    uint32_t n = read_word(h, h->s.counters + 3, &st);
    if (st != MG_OK) return st;
    d->size += n;
    return MG_OK;
}

mg_status mg_mlp_fit_normalization(mg_mlp m, mg_dataset d) {
    if (!m || !d || d->size == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_fit_normalization");
    cudaError_t e = mg::mlp_fit_norm(&m->m, d->dx, d->dy, d->size);
    if (e == cudaSuccess) e = mg::mlp_refresh_inference(&m->m);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_mlp_fit_normalization");
}

mg_status mg_mlp_train(mg_mlp m, mg_dataset d, uint32_t steps, uint32_t batch, float lr,
                       uint64_t seed, float* loss_curve) {
    if (!m || !d || d->size == 0 || batch == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_mlp_train");
    cudaError_t e = mg::mlp_train(&m->m, d->dx, d->dy, d->size, steps, batch, lr, seed, loss_curve);
    return e == cudaSuccess ? MG_OK : mlp_fail(e, "mg_mlp_train");
}

mg_status mg_set_surrogate(mg_handle h, mg_mlp m, uint32_t judge_period, uint32_t judge_stride,
                           float threshold) {
    if (!h) return fail(nullptr, MG_ERR_INVALID_ARG, "handle is NULL");
    if (h->n_inst && m) return packed_flags_ok(h, MG_STEP_SURROGATE);
    clear_graphs(h);
    if (!m) {
        h->sur = nullptr;
        return MG_OK;
    }
    if (!h->feat) {
        cudaError_t e = cudaMalloc(&h->feat, sizeof(__nv_bfloat16) * (size_t)h->cap * mg::MLP_IN);
        if (e == cudaSuccess) e = cudaMalloc(&h->feat_scale, 4ull * h->cap);
        if (e == cudaSuccess) e = cudaMalloc(&h->conc_plain, 4ull * h->cap * NTF);
        if (e == cudaSuccess) e = cudaMalloc(&h->sur_stats, 16);
        if (e != cudaSuccess) return fail(h, MG_ERR_OOM, "surrogate buffers");
    }
    {
        cudaError_t e = mg::make_feat_map(h->feat, h->cap, &h->feat_map);
        if (e != cudaSuccess) {
            h->sur = nullptr;
            return cuda_fail(h, e, "surrogate feature tensor map");
        }
    }
    MG_CUDA(h, cudaMemsetAsync(h->sur_stats, 0, 16, h->stream));
    cudaStreamSynchronize(m->st);
    h->sur = &m->m;
    h->judge_period = judge_period;
    h->judge_stride = judge_stride;
    h->judge_threshold = threshold;
    return check_device(h);
}

mg_status mg_surrogate_stats(mg_handle h, uint64_t* judged, uint64_t* handed_over, float* worst,
                             int32_t reset) {
    if (!h || !h->sur_stats) return fail(h, MG_ERR_INVALID_ARG, "no surrogate attached");
    uint32_t v[4] = {0, 0, 0, 0};
    MG_CUDA(h, cudaMemcpyAsync(v, h->sur_stats, 16, cudaMemcpyDeviceToHost, h->stream));
    MG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (judged) *judged = v[0];
    if (handed_over) *handed_over = v[1];
    if (worst) std::memcpy(worst, &v[2], 4);
    if (reset) MG_CUDA(h, cudaMemsetAsync(h->sur_stats, 0, 16, h->stream));
    return check_device(h);
}

// Number of kernels launched by mg_step since the handle was created.
uint64_t mg_kernel_launches(mg_handle h) { return h ? h->launches : 0; }

mg_status mg_device_bytes(mg_handle h, size_t* arena, size_t* total) {
    if (!h || !arena || !total) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    const size_t n = h->cap, C = (size_t)h->P.cells;
    size_t t = h->arena_bytes + h->staging_bytes;
    if (h->dense) t += 4 * (2 * C * NG + n * NG + NG);
    if (h->feat) t += sizeof(__nv_bfloat16) * n * mg::MLP_IN + 4 * n + 4 * n * NTF + 16;
    *arena = h->arena_bytes;
    *total = t;
    return MG_OK;
}

// ---- autotuner --------------------------------------------------------------------------------
// Times launch shapes on the handle's own state: each candidate runs `steps` graph steps from a
// snapshot of the whole arena, which is restored afterwards, so tuning leaves the simulation
// where it was.  First the density pass's shape (warps per block, search groups, sub-cell
// bits, search), then, one pass at a time with that shape, the block sizes of the force,
// gather and advance passes.  Results do not depend on the choice.
mg_status mg_autotune(mg_handle h, uint32_t steps, uint32_t flags, int32_t* choice, float* ms_per_step) {
    if (!h || steps == 0) return fail(h, MG_ERR_INVALID_ARG, "mg_autotune: bad arguments");
    if (flags & (MG_STEP_SURROGATE | MG_STEP_REMODEL))
        return fail(h, MG_ERR_INVALID_ARG, "mg_autotune times plain steps (physics and genes flags)");
    if (h->profile) return fail(h, MG_ERR_INVALID_ARG, "mg_autotune: profiling is on");
    if (h->search == 0) return fail(h, MG_ERR_INVALID_ARG, "mg_autotune tunes the warp searches (1, 2)");
    const int search0 = h->search;
    void* snap = nullptr;
    if (cudaMalloc(&snap, h->arena_bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, MG_ERR_OOM, "mg_autotune: no room for a snapshot of the arena");
    }
    struct Host {
        int cur, conc_cur, phase, osp;
        bool ever_sorted, brk_pending, flist_valid, reorigin_due;
        float time;
        uint64_t launches;
        uint32_t since_reorigin;
    };
    const Host saved{h->cur, h->conc_cur, h->phase, h->osp, h->ever_sorted, h->brk_pending, h->flist_valid,
                     h->reorigin_due, h->time, h->launches, h->since_reorigin};
    const DevParams P0 = h->P;
    auto restore = [&]() -> cudaError_t {
        h->cur = saved.cur; h->conc_cur = saved.conc_cur; h->phase = saved.phase;
        h->ever_sorted = saved.ever_sorted; h->brk_pending = saved.brk_pending;
        h->flist_valid = saved.flist_valid; h->time = saved.time; h->launches = saved.launches;
        if (h->osp != saved.osp) swap_ospace(h);
        h->reorigin_due = saved.reorigin_due;
        h->since_reorigin = saved.since_reorigin;
        return cudaMemcpyAsync(h->arena, snap, h->arena_bytes, cudaMemcpyDeviceToDevice, h->stream);
    };
    mg_status st = MG_OK;
    cudaError_t e = cudaMemcpyAsync(snap, h->arena, h->arena_bytes, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) st = cuda_fail(h, e, "mg_autotune snapshot");
    cudaEvent_t a = nullptr, z = nullptr;
    if (st == MG_OK && (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&z) != cudaSuccess))
        st = fail(h, MG_ERR_CUDA, "mg_autotune: events");
    // one trial of the shape in h->P / h->search: two warm steps capture the graphs of both
    // buffer parities, then the timed run, each from the snapshot
    auto trial = [&](float* t) -> mg_status {
        clear_graphs(h);
        cudaError_t e2;
        if ((e2 = restore()) != cudaSuccess) return cuda_fail(h, e2, "mg_autotune restore");
        mg_status s2 = run_steps(h, 2, flags);
        if (s2 != MG_OK) return s2;
        if ((e2 = restore()) != cudaSuccess) return cuda_fail(h, e2, "mg_autotune restore");
        cudaEventRecord(a, h->stream);
        if ((s2 = run_steps(h, steps, flags)) != MG_OK) return s2;
        cudaEventRecord(z, h->stream);
        cudaEventSynchronize(z);
        *t = 0.f;
        cudaEventElapsedTime(t, a, z);
        return MG_OK;
    };
    struct Cand { int warps, group, sub, search; };
    const bool fine_ok = h->P.gsrch == 3;
    const Cand cands[] = {{8, 0, 2, 1}, {8, 1, 2, 1}, {8, 0, 1, 1}, {8, 1, 1, 1}, {4, 0, 2, 1},
                          {4, 1, 2, 1}, {4, 0, 1, 1}, {4, 1, 1, 1}, {8, 0, 1, 2}, {4, 0, 1, 2}};
    float best = 0.f;
    Cand pick = cands[0];
    for (const Cand& c : cands) {
        if (st != MG_OK) break;
        if (c.search == 2 && (!fine_ok || h->n_inst)) continue;
        h->search = c.search;
        h->P.dens_warps = c.warps;
        h->P.group_mode = c.group;
        h->P.sub_bits = c.sub;
        float t = 0.f;
        if ((st = trial(&t)) != MG_OK) break;
        // the first candidate (the default shape) stays unless another beats the best by 3%:
        // on fresh states several shapes time within noise, and the default holds up best as
        // the tissue evolves
        if (&c == cands || t < best * 0.97f) { best = t; pick = c; }
    }
    // block sizes of the one-particle-per-thread passes, one pass at a time, the density
    // shape fixed at its pick (its time with 256-thread blocks is the time to beat)
    int threads[3] = {P0.force_threads, P0.gather_threads, P0.advance_threads};
    if (st == MG_OK) {
        h->search = pick.search;
        h->P.dens_warps = pick.warps;
        h->P.group_mode = pick.group;
        h->P.sub_bits = pick.sub;
        int* slot[3] = {&h->P.force_threads, &h->P.gather_threads, &h->P.advance_threads};
        for (int k = 0; k < 3 && st == MG_OK; k++) {
            const int keep = *slot[k];
            for (int nt : {128, 256, 512}) {
                if (nt == keep) continue;
                *slot[k] = nt;
                float t = 0.f;
                if ((st = trial(&t)) != MG_OK) break;
                if (t < best * 0.97f) { best = t; threads[k] = nt; }
            }
            *slot[k] = threads[k];
        }
    }
    if (a) cudaEventDestroy(a);
    if (z) cudaEventDestroy(z);
    h->P = P0;
    h->search = search0;
    if (st == MG_OK) {
        h->P.dens_warps = pick.warps;
        h->P.group_mode = pick.group;
        h->P.sub_bits = pick.sub;
        h->search = pick.search;
        h->P.force_threads = threads[0];
        h->P.gather_threads = threads[1];
        h->P.advance_threads = threads[2];
    }
    clear_graphs(h);
    e = restore();
    h->flist_valid = false;
    // the fine-cell search reads sub-cell tables that only a sort made for it writes
    if (h->search == 2 && search0 != 2 && h->phase == PHASE_SORTED) h->phase = PHASE_UNSORTED;
    cudaStreamSynchronize(h->stream);
    cudaFree(snap);
    if (st != MG_OK) return st;
    if (e != cudaSuccess) return cuda_fail(h, e, "mg_autotune restore");
    if (choice) { choice[0] = pick.warps; choice[1] = pick.group; choice[2] = pick.sub; choice[3] = pick.search; }
    if (ms_per_step) *ms_per_step = best / (float)steps;
    return check_device(h);
}

mg_status mg_get_block_sizes(mg_handle h, int32_t* threads) {
    if (!h || !threads) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    threads[0] = h->P.force_threads;
    threads[1] = h->P.gather_threads;
    threads[2] = h->P.advance_threads;
    return MG_OK;
}

mg_status mg_set_block_sizes(mg_handle h, const int32_t* threads) {
    if (!h || !threads) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    for (int k = 0; k < 3; k++)
        if (threads[k] != 128 && threads[k] != 256 && threads[k] != 512)
            return fail(h, MG_ERR_INVALID_ARG, "block sizes: 128, 256 or 512 threads");
    h->P.force_threads = threads[0];
    h->P.gather_threads = threads[1];
    h->P.advance_threads = threads[2];
    clear_graphs(h);
    return MG_OK;
}

mg_status mg_get_tuning(mg_handle h, int32_t* choice) {
    if (!h || !choice) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    choice[0] = h->P.dens_warps;
    choice[1] = h->P.group_mode;
    choice[2] = h->P.sub_bits;
    choice[3] = h->search;
    return MG_OK;
}

mg_status mg_set_tuning(mg_handle h, const int32_t* choice) {
    if (!h || !choice) return fail(h, MG_ERR_INVALID_ARG, "NULL argument");
    if ((choice[0] != 4 && choice[0] != 8) || (choice[1] != 0 && choice[1] != 1) ||
        (choice[2] != 1 && choice[2] != 2) || choice[3] < 0 || choice[3] > 2)
        return fail(h, MG_ERR_INVALID_ARG,
                    "tuning: warps 4 or 8, group mode 0 or 1, sub-cell bits 1 or 2, search 0-2");
    if (choice[3] == 2 && (choice[2] != 1 || h->P.gsrch != 3))
        return fail(h, MG_ERR_INVALID_ARG, "the fine-cell search needs sub-cell bits 1 and gsrch 3");
    if (h->n_inst && choice[3] != 1)
        return fail(h, MG_ERR_UNSUPPORTED, "packed instances use the warp-cooperative search (1)");
    if (choice[3] == 2 && (h->search != 2 || h->P.sub_bits != 1) && h->phase == PHASE_SORTED)
        h->phase = PHASE_UNSORTED;  // the fine-cell search needs a sort made for it
    h->P.dens_warps = choice[0];
    h->P.group_mode = choice[1];
    h->P.sub_bits = choice[2];
    h->search = choice[3];
    h->flist_valid = false;
    clear_graphs(h);
    return MG_OK;
}

// ---- failure-detection self-test ---------------------------------------------------------------
mg_status mg_selftest_bounded_wait(int32_t which, uint32_t spin_limit) {
    if (which < 0 || which > 2 || spin_limit == 0 || spin_limit > (1u << 20))
        return fail(nullptr, MG_ERR_INVALID_ARG, "mg_selftest_bounded_wait: which must be 0, 1 or 2, spin_limit 1 .. 1048576");
    cudaStream_t st = nullptr;
    MG_CUDA(nullptr, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    uint32_t bits = 0;
    cudaError_t e = which == 0 ? mg::scan_selftest_wait_timeout(spin_limit, &bits, st)
                  : which == 1 ? mg::mlp_selftest_wait_timeout(spin_limit, &bits, st)
                               : mg::mlp_selftest_gemm_wait_timeout(spin_limit, &bits, st);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "mg_selftest_bounded_wait");
    const uint32_t expect = which == 0 ? (uint32_t)ERR_SCAN_TIMEOUT : (uint32_t)mg::MLP_ERR_MBAR_TIMEOUT;
    static const char* const what[3] = {
        "self-test: prefix-sum look-back gave up waiting (bounded spin)",
        "self-test: tensor-core completion wait gave up (bounded spin)",
        "self-test: training-GEMM completion wait gave up (bounded spin)"};
    if (bits & expect) return fail(nullptr, MG_ERR_DEVICE_TIMEOUT, what[which]);
    return MG_OK;
}

// ---- batched instances -----------------------------------------------------------------------
static void batch_clear_graphs(mg_batch b) {
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

mg_status mg_batch_create(const mg_handle* hs, uint32_t count, mg_batch* out) {
    if (!hs || !out || count == 0) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_batch_create: bad arguments");
    for (uint32_t k = 0; k < count; k++) {
        if (!hs[k]) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_batch_create: NULL member");
        for (uint32_t q = 0; q < k; q++)
            if (hs[q] == hs[k]) return fail(nullptr, MG_ERR_INVALID_ARG, "mg_batch_create: a member appears twice");
        if (hs[k]->device != hs[0]->device)
            return fail(nullptr, MG_ERR_INVALID_ARG, "mg_batch_create: members on different devices");
    }
    mg_batch b = new mg_batch_s();
    b->hs.assign(hs, hs + count);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (b->stream) cudaStreamDestroy(b->stream);
        delete b;
        return cuda_fail(nullptr, e, "mg_batch_create");
    }
    *out = b;
    return MG_OK;
}

mg_status mg_batch_destroy(mg_batch b) {
    if (!b) return MG_OK;
    cudaStreamSynchronize(b->stream);
    batch_clear_graphs(b);
    cudaEventDestroy(b->done);
    cudaStreamDestroy(b->stream);
    delete b;
    return MG_OK;
}

static mg_status batch_graph(mg_batch b, uint32_t flags, cudaGraphExec_t* out) {
    std::vector<uint64_t> epochs;
    for (mg_system* h : b->hs) epochs.push_back(h->graph_epoch);
    if (epochs != b->epochs) {  // a member changed since the cached graphs were captured
        batch_clear_graphs(b);
        b->epochs = epochs;
    }
    std::string key = std::to_string(flags) + ":";
    for (mg_system* h : b->hs) key += (char)('0' + 4 * h->osp + 2 * h->cur + h->conc_cur);
    auto it = b->graphs.find(key);
    if (it != b->graphs.end()) {
        for (mg_system* h : b->hs) advance_state(h, flags);
        *out = it->second;
        return MG_OK;
    }
    cudaGraph_t bg = nullptr;
    MG_CUDA(nullptr, cudaGraphCreate(&bg, 0));
    // Members run in groups of MG_BATCH_GROUP (32): a group's steps are independent branches, and an
    // empty node joins each group before the next starts.  One flat level of hundreds of
    // branches schedules far worse than a few levels of tens (measured: 256 members of 1,000
    // particles take 11x the time of 64; groups of 32 were fastest among 16-256).
    cudaGraphNode_t join = nullptr;
    std::vector<cudaGraphNode_t> group;
    std::vector<std::pair<int, int>> state0;  // members' buffer states before the capture
    for (mg_system* h : b->hs) state0.emplace_back(h->cur, h->conc_cur);
    auto restore = [&] {
        for (size_t k = 0; k < b->hs.size(); k++) {
            b->hs[k]->cur = state0[k].first;
            b->hs[k]->conc_cur = state0[k].second;
        }
    };
    size_t m = 0;
    for (mg_system* h : b->hs) {
        if (group.size() == (size_t)MG_BATCH_GROUP) {
            cudaGraphNode_t j = nullptr;
            cudaError_t e = cudaGraphAddEmptyNode(&j, bg, group.data(), group.size());
            if (e != cudaSuccess) {
                cudaGraphDestroy(bg);
                restore();
                return cuda_fail(nullptr, e, "batch group join");
            }
            join = j;
            group.clear();
        }
        m++;
        DevParams saved = h->P;
        if (flags & MG_STEP_FREEZE) h->P.freeze = 1;
        cudaGraph_t g = nullptr;
        prepare_step(h, flags);
        cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue_step(h, flags, false);  // advances the member's buffer state
            e = cudaStreamEndCapture(h->stream, &g);
        }
        h->P = saved;
        cudaGraphNode_t node;
        if (e == cudaSuccess) e = cudaGraphAddChildGraphNode(&node, bg, join ? &join : nullptr, join ? 1 : 0, g);
        if (e == cudaSuccess) group.push_back(node);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGraphDestroy(bg);
            restore();
            return cuda_fail(h, e, "batch step capture");
        }
    }
    cudaGraphExec_t ge = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ge, bg, 0);
    cudaGraphDestroy(bg);
    if (e != cudaSuccess) {
        restore();
        return cuda_fail(nullptr, e, "cudaGraphInstantiate (batch)");
    }
    b->graphs[key] = ge;
    *out = ge;
    return MG_OK;
}

static mg_status batch_run(mg_batch b, uint32_t nsteps, uint32_t flags, float* ms) {
    if (!b) return fail(nullptr, MG_ERR_INVALID_ARG, "batch is NULL");
    for (mg_system* h : b->hs) {
        if (h->profile) return fail(h, MG_ERR_INVALID_ARG, "batch members must not be profiling");
        if ((flags & MG_STEP_SURROGATE) && !h->sur)
            return fail(h, MG_ERR_INVALID_ARG, "surrogate step without an attached network (mg_set_surrogate)");
        MG_CUDA(h, cudaStreamSynchronize(h->stream));  // members' earlier work first
    }
    cudaEvent_t a = nullptr, z = nullptr;
    if (ms) {
        MG_CUDA(nullptr, cudaEventCreate(&a));
        MG_CUDA(nullptr, cudaEventCreate(&z));
        MG_CUDA(nullptr, cudaEventRecord(a, b->stream));
    }
    mg_status st = MG_OK;
    uint32_t launched = 0;  // steps whose graph was launched
    for (uint32_t s = 0; s < nsteps && st == MG_OK; s++) {
        cudaGraphExec_t ge = nullptr;
        st = batch_graph(b, flags, &ge);
        if (st == MG_OK) {
            cudaError_t e = cudaGraphLaunch(ge, b->stream);
            if (e != cudaSuccess) {
                st = cuda_fail(nullptr, e, "cudaGraphLaunch (batch)");
                for (mg_system* h : b->hs) undo_state(h, flags);  // the step did not run
            } else {
                launched++;
            }
        }
    }
    if (ms) {
        cudaEventRecord(z, b->stream);
        cudaEventSynchronize(z);
        float t = 0.f;
        cudaEventElapsedTime(&t, a, z);
        *ms = t;
        cudaEventDestroy(a);
        cudaEventDestroy(z);
    }
    // later work on a member's own stream waits for the batch
    cudaEventRecord(b->done, b->stream);
    for (mg_system* h : b->hs) {
        cudaStreamWaitEvent(h->stream, b->done, 0);
        if (launched) after_steps(h, launched, flags);
    }
    if (st != MG_OK) return st;
    for (mg_system* h : b->hs) {
        mg_status s2 = check_device(h);
        if (s2 != MG_OK) return s2;
    }
    return MG_OK;
}

mg_status mg_batch_step(mg_batch b, uint32_t nsteps, uint32_t flags) {
    return batch_run(b, nsteps, flags, nullptr);
}

mg_status mg_batch_time_steps(mg_batch b, uint32_t nsteps, uint32_t flags, float* ms) {
    if (!ms) return fail(nullptr, MG_ERR_INVALID_ARG, "NULL argument");
    return batch_run(b, nsteps, flags, ms);
}

}  // extern "C"

mg_status mg::record_thread_error(mg_status st, const char* msg) { return fail(nullptr, st, msg); }
