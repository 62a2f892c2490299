/*
 * mg_fluid_system.hpp - header-only C++ host class over mg_abi.h with the method names of the
 * reference's FluidSystem (Morphogenesis src/fluid_system.h:357-766), for a host program that
 * wants the reference's calling sequence on this library:
 *
 *     mg::FluidSystem fs;
 *     fs.FluidSetupCL(num, gsrch, res, size, delta, gmin, gmax, total, chk);   // host_CL.cpp:39
 *     fs.FluidParamCL(ss, sr, pr, mass, rest, bmin, bmax, estiff, istiff, visc, surface_t,
 *                     damp, fmin, fmax, ffreq, gslope, gx, gy, gz, al, vl, a_f, a_p);
 *                                                                  // fluid_system.cpp:521
 *     fs.UpdateGenome(genome);                                     // fluid_system.cpp:494
 *     fs.AllocateParticles();          // AllocateParticles / AllocateGrid: device + host buffers
 *     ... fill fs.mcpu(FPOS) etc. (getPos(i), getConc(tf), ...) ...
 *     fs.TransferToCL();
 *     fs.Run2PhysicalSort(); fs.Run2InnerPhysicalLoop(); fs.Run2GeneAction(); ...
 *     fs.TransferFromCL();
 *
 * The host buffers (the reference's m_Fluid.mcpu[id], fluid.h:239-242) hold the reference
 * layouts of mg_abi.h, with FCONC species-major as the reference host keeps it
 * (getConc(tf) = FCONC + tf * mMaxPoints, fluid_system.h:574).  Errors are thrown as
 * mg::Error with the library's message (the reference prints and exits instead,
 * fluid_system.cpp:28-33).  One object per simulation, used from one host thread.
 */
#ifndef MG_FLUID_SYSTEM_HPP
#define MG_FLUID_SYSTEM_HPP

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mg_abi.h"

namespace mg {

class Error : public std::runtime_error {
   public:
    Error(mg_status status, const std::string& what) : std::runtime_error(what), status(status) {}
    mg_status status;
};

class FluidSystem {
   public:
    FluidSystem() = default;
    ~FluidSystem() { mg_destroy(h_); }
    FluidSystem(const FluidSystem&) = delete;
    FluidSystem& operator=(const FluidSystem&) = delete;
    FluidSystem(FluidSystem&& o) noexcept { *this = std::move(o); }
    FluidSystem& operator=(FluidSystem&& o) noexcept {
        if (this != &o) {
            mg_destroy(h_);
            p_ = o.p_;
            g_ = o.g_;
            h_ = o.h_;
            max_points_ = o.max_points_;
            for (int k = 0; k < MG_MAX_BUF; k++) mcpu_[k] = std::move(o.mcpu_[k]);
            o.h_ = nullptr;
        }
        return *this;
    }

    // ---- set-up -------------------------------------------------------------------------
    // FluidSetupCL (host_CL.cpp:39-106): particle capacity and grid.  The derived gridAdj and
    // gridScanMax are computed by the library.
    void FluidSetupCL(int num, int gsrch, const int res[3], const float size[3], const float delta[3],
                      const float gmin[3], const float gmax[3], int total, int /*chk*/) {
        max_points_ = (uint32_t)num;
        p_.grid_srch = gsrch;
        for (int k = 0; k < 3; k++) {
            p_.grid_res[k] = res[k];
            p_.grid_size[k] = size[k];
            p_.grid_delta[k] = delta[k];
            p_.grid_min[k] = gmin[k];
            p_.grid_max[k] = gmax[k];
        }
        p_.grid_total = total;
    }
    // FluidParamCL (fluid_system.cpp:521-610); on an allocated system it updates the parameters
    // (UpdateParams).
    void FluidParamCL(float ss, float sr, float pr, float mass, float rest, const float bmin[3],
                      const float bmax[3], float estiff, float istiff, float visc, float surface_t,
                      float damp, float fmin, float fmax, float ffreq, float gslope, float gx, float gy,
                      float gz, float al, float vl, float a_f, float a_p) {
        p_.psimscale = ss;
        p_.psmoothradius = sr;
        p_.pradius = pr;
        p_.pmass = mass;
        p_.prest_dens = rest;
        for (int k = 0; k < 3; k++) {
            p_.pboundmin[k] = bmin[k];
            p_.pboundmax[k] = bmax[k];
        }
        p_.pextstiff = estiff;
        p_.pintstiff = istiff;
        p_.pvisc = visc;
        p_.psurface_t = surface_t;
        p_.pdamp = damp;
        p_.pforce_min = fmin;
        p_.pforce_max = fmax;
        p_.pforce_freq = ffreq;
        p_.pground_slope = gslope;
        p_.pgravity[0] = gx;
        p_.pgravity[1] = gy;
        p_.pgravity[2] = gz;
        p_.paccel_limit = al;
        p_.pvel_limit = vl;
        p_.actuation_factor = a_f;
        p_.actuation_period = a_p;
        if (h_) check(mg_update_params(h_, &p_), "FluidParamCL");
    }
    // m_DT and m_Time (fluid_system.h), applied at allocation or through SetParam afterwards
    void SetTimeStep(float dt) {
        p_.dt = dt;
        if (h_) SetParam(MG_PDT, dt);
    }
    void SetTime(float t) {
        p_.time = t;
        if (h_) SetParam(MG_PTIME, t);
    }
    // UpdateGenome (fluid_system.cpp:494)
    void UpdateGenome(const mg_genome& g) {
        g_ = g;
        if (h_) check(mg_update_genome(h_, &g_), "UpdateGenome");
    }
    // AllocateParticles + AllocateGrid (host_CL.cpp:107-174): the device system and the host
    // buffers of every exchanged id, zeroed.
    void AllocateParticles() {
        if (h_) throw Error(MG_ERR_INVALID_ARG, "AllocateParticles: already allocated");
        check(mg_create(&p_, &g_, max_points_, &h_), "AllocateParticles");
        check(mg_set_option(h_, MG_OPT_CONC_LAYOUT, 1), "AllocateParticles");
        for (int id : kHostBufs) {
            size_t n = 0;
            check(mg_buffer_bytes(h_, id, &n), "AllocateParticles");
            mcpu_[id].assign(n / sizeof(uint32_t), 0u);  // every exchanged layout is 32-bit words
        }
    }
    // SetParam (fluid_system.h:77-104 ids, plus MG_PDT / MG_PTIME / MG_PFREEZE)
    void SetParam(int id, float v) { check(mg_set_param(h_, id, v), "SetParam"); }

    // ---- host buffers -------------------------------------------------------------------
    void* mcpu(int id) { return mcpu_[id].empty() ? nullptr : mcpu_[id].data(); }
    size_t mcpu_bytes(int id) const { return mcpu_[id].size() * sizeof(uint32_t); }
    float* getPos(int i) { return f(MG_FPOS) + 4 * (size_t)i; }
    float* getVel(int i) { return f(MG_FVEL) + 4 * (size_t)i; }
    float* getVeval(int i) { return f(MG_FVEVAL) + 4 * (size_t)i; }
    uint32_t* getElastIdx(int i) { return u(MG_FELASTIDX) + (size_t)MG_BOND_DATA * i; }
    uint32_t* getParticle_Idx(int i) { return u(MG_FPARTICLEIDX) + 2 * (size_t)MG_BONDS_PER_PARTICLE * i; }
    uint32_t* getParticle_ID(int i) { return u(MG_FPARTICLE_ID) + (size_t)i; }
    float* getConc(int tf) { return f(MG_FCONC) + (size_t)tf * max_points_; }
    uint32_t* getEpiGen(int gene) { return u(MG_FEPIGEN) + (size_t)gene * max_points_; }
    uint32_t MaxPoints() const { return max_points_; }
    uint32_t NumPoints() const { return counts().first; }
    uint32_t ActivePoints() const { return counts().second; }
    float GetTime() const {
        float t = 0.f;
        mg_get_time(h_, &t);
        return t;
    }
    mg_handle handle() const { return h_; }

    // ---- transfer (host_CL.cpp:1521-1668) --------------------------------------------------
    void TransferToCL() {
        for (int id : kHostBufs)
            check(mg_upload(h_, id, mcpu_[id].data(), mcpu_bytes(id)), "TransferToCL");
    }
    void TransferFromCL() {
        for (int id : kHostBufs)
            check(mg_download(h_, id, mcpu_[id].data(), mcpu_bytes(id)), "TransferFromCL");
    }

    // ---- stages (the *CL wrappers of host_CL.cpp / host_CUDA.cpp) ------------------------------
    void InsertParticlesCL() { check(mg_insert_particles(h_), "InsertParticlesCL"); }
    void PrefixSumCellsCL() { check(mg_prefix_sum_cells(h_), "PrefixSumCellsCL"); }
    void CountingSortFullCL() { check(mg_counting_sort_full(h_), "CountingSortFullCL"); }
    void ComputePressureCL() { check(mg_compute_pressure(h_), "ComputePressureCL"); }
    void ComputeForceCL() { check(mg_compute_force(h_), "ComputeForceCL"); }
    void ComputeDiffusionCL() { check(mg_compute_diffusion(h_), "ComputeDiffusionCL"); }
    void ComputeGenesCL() { check(mg_compute_genes(h_), "ComputeGenesCL"); }
    void ComputeBondChangesCL(uint32_t steps) { check(mg_compute_bond_changes(h_, steps), "ComputeBondChangesCL"); }
    void ComputeParticleChangesCL() { check(mg_run_remodelling(h_), "ComputeParticleChangesCL"); }
    void AdvanceCL() { check(mg_advance(h_), "AdvanceCL"); }
    void ZeroVelCL() { check(mg_zero_vel(h_), "ZeroVelCL"); }

    // ---- run loop (fluid_system.cpp:1179-1349, 1919-2071) ------------------------------------
    void Run2PhysicalSort() { check(mg_run_physical_sort(h_), "Run2PhysicalSort"); }
    void Run2InnerPhysicalLoop() { check(mg_run_inner_physical_loop(h_), "Run2InnerPhysicalLoop"); }
    void Run2GeneAction() { check(mg_run_gene_action(h_), "Run2GeneAction"); }
    void Run2Remodelling(uint32_t steps_per_inner_loop) {
        check(mg_run_remodelling_steps(h_, steps_per_inner_loop), "Run2Remodelling");
    }
    // the legacy Run() order, nsteps steps (one sort per step)
    void Run(uint32_t nsteps = 1, uint32_t flags = MG_STEP_DEFAULT) { check(mg_step(h_, nsteps, flags), "Run"); }

    // ---- tuning (results are identical for every choice) ---------------------------------------
    // Times the launch shapes and block sizes over `steps` steps of the current state (restored
    // afterwards) and keeps the fastest; returns its ms per step.  Call after TransferToCL.
    float Autotune(uint32_t steps = 5, uint32_t flags = MG_STEP_DEFAULT) {
        int32_t choice[4];
        float ms = 0.f;
        check(mg_autotune(h_, steps, flags, choice, &ms), "Autotune");
        return ms;
    }
    // threads per block of the force, gather and advance passes: 128, 256 or 512 each
    void SetBlockSizes(int32_t force, int32_t gather, int32_t advance) {
        const int32_t t[3] = {force, gather, advance};
        check(mg_set_block_sizes(h_, t), "SetBlockSizes");
    }
    // MG_OPT_* (include/mg_abi.h)
    void SetOption(int32_t option, int32_t value) { check(mg_set_option(h_, option, value), "SetOption"); }

   private:
    static constexpr int kHostBufs[] = {MG_FPOS, MG_FVEL, MG_FVEVAL, MG_FFORCE, MG_FPRESS, MG_FDENSITY,
                                        MG_FAGE, MG_FCOLOR, MG_FELASTIDX, MG_FPARTICLEIDX, MG_FPARTICLE_ID,
                                        MG_FMASS_RADIUS, MG_FNERVEIDX, MG_FCONC, MG_FEPIGEN};
    float* f(int id) { return reinterpret_cast<float*>(mcpu_[id].data()); }
    uint32_t* u(int id) { return reinterpret_cast<uint32_t*>(mcpu_[id].data()); }
    std::pair<uint32_t, uint32_t> counts() const {
        uint32_t a = 0, b = 0;
        mg_get_counts(h_, &a, &b);
        return {a, b};
    }
    void check(mg_status s, const char* where) const {
        if (s != MG_OK) throw Error(s, std::string(where) + ": " + (mg_last_error(h_) ? mg_last_error(h_) : ""));
    }

    mg_fparams p_{};
    mg_genome g_{};
    mg_handle h_ = nullptr;
    uint32_t max_points_ = 0;
    std::vector<uint32_t> mcpu_[MG_MAX_BUF];
};

}  // namespace mg

#endif  // MG_FLUID_SYSTEM_HPP
