// abi_host.cpp - a compiled C++ host on include/mg_fluid_system.hpp (the FluidSystem-style
// façade over mg_abi.h), driving the reference's calling sequence: FluidSetupCL, FluidParamCL,
// UpdateGenome, AllocateParticles, buffers filled through the host mirrors, TransferToCL, the
// tuning calls (re-origin period, block sizes, autotune: none may change a result), one
// Run2 cycle (Run2PhysicalSort, Run2InnerPhysicalLoop, Run2GeneAction), `steps` legacy steps,
// TransferFromCL.  Built and run by tests/test_cpp_host.py, which compares what it writes with
// the same sequence run through the Python binding.
//
//   abi_host DIR STEPS
// DIR holds params.bin (an mg_fparams), genome.bin (an mg_genome), n.txt (particles) and
// in_<id>.bin per uploaded buffer (reference layouts, FCONC species-major); the host writes
// out_<id>.bin for the same ids.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mg_fluid_system.hpp"

namespace {

std::vector<char> slurp(const std::string& path) {
    std::vector<char> out;
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return out;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out.insert(out.end(), buf, buf + n);
    std::fclose(f);
    return out;
}

bool spill(const std::string& path, const void* data, size_t bytes) {
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, bytes, f) == bytes;
    return std::fclose(f) == 0 && ok;
}

const int kIds[] = {MG_FPOS, MG_FVEL, MG_FVEVAL, MG_FELASTIDX, MG_FPARTICLEIDX, MG_FPARTICLE_ID,
                    MG_FCONC, MG_FEPIGEN};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: abi_host DIR STEPS\n");
        return 2;
    }
    const std::string dir = argv[1];
    const unsigned steps = (unsigned)std::strtoul(argv[2], nullptr, 10);
    const std::vector<char> pb = slurp(dir + "/params.bin"), gb = slurp(dir + "/genome.bin");
    const std::vector<char> nb = slurp(dir + "/n.txt");
    if (pb.size() != sizeof(mg_fparams) || gb.size() != sizeof(mg_genome) || nb.empty()) {
        std::fprintf(stderr, "abi_host: bad inputs in %s\n", dir.c_str());
        return 2;
    }
    mg_fparams p;
    mg_genome g;
    std::memcpy(&p, pb.data(), sizeof p);
    std::memcpy(&g, gb.data(), sizeof g);
    const int n = std::atoi(std::string(nb.begin(), nb.end()).c_str());
    try {
        mg::FluidSystem fs;
        fs.FluidSetupCL(n, p.grid_srch, p.grid_res, p.grid_size, p.grid_delta, p.grid_min, p.grid_max,
                        p.grid_total, 0);
        fs.FluidParamCL(p.psimscale, p.psmoothradius, p.pradius, p.pmass, p.prest_dens, p.pboundmin,
                        p.pboundmax, p.pextstiff, p.pintstiff, p.pvisc, p.psurface_t, p.pdamp,
                        p.pforce_min, p.pforce_max, p.pforce_freq, p.pground_slope, p.pgravity[0],
                        p.pgravity[1], p.pgravity[2], p.paccel_limit, p.pvel_limit,
                        p.actuation_factor, p.actuation_period);
        fs.SetTimeStep(p.dt);
        fs.SetTime(p.time);
        fs.UpdateGenome(g);
        fs.AllocateParticles();
        for (int id : kIds) {
            const std::vector<char> b = slurp(dir + "/in_" + std::to_string(id) + ".bin");
            if (b.size() != fs.mcpu_bytes(id)) {
                std::fprintf(stderr, "abi_host: in_%d.bin has %zu bytes, expected %zu\n", id, b.size(),
                             fs.mcpu_bytes(id));
                return 2;
            }
            std::memcpy(fs.mcpu(id), b.data(), b.size());
        }
        // the species-major accessor sees species tf of particle i where the reference's does
        if (fs.getConc(3)[5] != reinterpret_cast<const float*>(fs.mcpu(MG_FCONC))[3 * n + 5]) return 3;
        fs.TransferToCL();
        // tuning changes no result: the run below must match the Python binding's defaults
        fs.SetOption(MG_OPT_REORIGIN_PERIOD, 3);
        fs.SetBlockSizes(512, 128, 256);
        if (!(fs.Autotune(2) > 0.f)) return 5;
        fs.Run2PhysicalSort();
        fs.Run2InnerPhysicalLoop();
        fs.Run2GeneAction();
        fs.Run(steps);
        fs.TransferFromCL();
        for (int id : kIds)
            if (!spill(dir + "/out_" + std::to_string(id) + ".bin", fs.mcpu(id), fs.mcpu_bytes(id))) return 4;
        std::printf("abi_host: %u particles, %u active, time %.6f\n", fs.NumPoints(), fs.ActivePoints(),
                    (double)fs.GetTime());
    } catch (const mg::Error& e) {
        std::fprintf(stderr, "abi_host: %s (status %d)\n", e.what(), (int)e.status);
        return 1;
    }
    return 0;
}
