// mg_files.cpp - the reference's file formats: SimParams.txt, genome.csv, the particle CSV written
// by SavePointsCSV2 (with the parameter set-up ReadPointsCSV2 performs), SpecificationFile.txt,
// results.csv and the VTP frames of SavePointsVTP2 (written as VTK XML without VTK).
//
// Reference: ReadSimParams / WriteSimParams (fileCL_IO.cpp:471-600), ReadGenome / WriteGenome
// (fileCL_IO.cpp:71-249), SavePointsCSV2 / ReadPointsCSV2 (fileCL_IO.cpp:250-469), SetupSpacing
// (fluid_system.cpp:2521-2546), UpdateParams (fluid_system.cpp:612-628).  The line layouts are
// the reference's, so files written by either side parse on the other.  Differences:
//  - errors are returned (the reference asserts or exits);
//  - the genome's sensitivity and transcription-factor rates are floats here (they are read with
//    %f, which also reads the reference's integers); mg_write_genome writes them as integers
//    (the reference format, values rounded) or as floats in the same layout;
//  - the points reader takes the file's own header counts and checks them against the sizes
//    this build uses.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mg_abi.h"
#include "mg_internal.cuh"

using namespace mg;

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

mg_status bad(const std::string& what) { return record_thread_error(MG_ERR_INVALID_ARG, what.c_str()); }

// Layout text between fields is matched and dropped, as the reference's readers do.
inline void skip(int) {}

}  // namespace

extern "C" {

mg_status mg_read_simparams(const char* path, mg_simparams* sp) {
    if (!path || !sp) return bad("mg_read_simparams: NULL argument");
    File fh(path, "rb");
    if (!fh.f) return bad(std::string("mg_read_simparams: cannot open ") + path);
    FILE* f = fh.f;
    mg_simparams s{};
    int ret = 0;
    ret += std::fscanf(f, " m_Time = %f\n ", &s.time);
    ret += std::fscanf(f, "m_DT = %f\n ", &s.dt);
    ret += std::fscanf(f, "m_Param [ PSIMSCALE ] = %f\n ", &s.simscale);
    ret += std::fscanf(f, "m_Param [ PGRID_DENSITY ] = %f\n ", &s.grid_density);
    ret += std::fscanf(f, "m_Param [ PVISC ] = %f\n ", &s.visc);
    ret += std::fscanf(f, "m_Param [ PSURFACE_TENSION ] = %f\n ", &s.surface_tension);
    ret += std::fscanf(f, "m_Param [ PRESTDENSITY ] = %f\n ", &s.rest_density);
    ret += std::fscanf(f, "m_Param [ PSPACING ] = %f\n ", &s.spacing);
    ret += std::fscanf(f, "m_Param [ PMASS ] = %f\n ", &s.mass);
    ret += std::fscanf(f, "m_Param [ PRADIUS ] = %f\n ", &s.radius);
    ret += std::fscanf(f, "m_Param [ PDIST ] = %f\n ", &s.dist);
    ret += std::fscanf(f, "m_Param [ PSMOOTHRADIUS ] = %f\n ", &s.smooth_radius);
    ret += std::fscanf(f, "m_Param [ PINTSTIFF ] = %f\n ", &s.intstiff);
    ret += std::fscanf(f, "m_Param [ PEXTSTIFF ] = %f\n ", &s.extstiff);
    ret += std::fscanf(f, "m_Param [ PEXTDAMP ] = %f\n ", &s.extdamp);
    ret += std::fscanf(f, "m_Param [ PACCEL_LIMIT ] = %f\n ", &s.accel_limit);
    ret += std::fscanf(f, "m_Param [ PVEL_LIMIT ] = %f\n ", &s.vel_limit);
    ret += std::fscanf(f, "m_Param [ PGRAV ] = %f\n ", &s.grav);
    ret += std::fscanf(f, "m_Param [ PGROUND_SLOPE ] = %f\n ", &s.ground_slope);
    ret += std::fscanf(f, "m_Param [ PFORCE_MIN ] = %f\n ", &s.force_min);
    ret += std::fscanf(f, "m_Param [ PFORCE_MAX ] = %f\n ", &s.force_max);
    ret += std::fscanf(f, "m_Param [ PFORCE_FREQ ] = %f\n ", &s.force_freq);
    ret += std::fscanf(f, "m_Vec [ PPLANE_GRAV_DIR ].Set ( %f, %f, %f )\n ", &s.plane_grav_dir[0],
                       &s.plane_grav_dir[1], &s.plane_grav_dir[2]);
    ret += std::fscanf(f, "// Default sim config\n ");
    ret += std::fscanf(f, "m_Param [ PGRIDSIZE ] = %f\n ", &s.grid_size);
    ret += std::fscanf(f, "m_Vec [ PVOLMIN ].Set ( %f, %f, %f )\n ", &s.volmin[0], &s.volmin[1], &s.volmin[2]);
    ret += std::fscanf(f, "m_Vec [ PVOLMAX ].Set ( %f, %f, %f )\n ", &s.volmax[0], &s.volmax[1], &s.volmax[2]);
    ret += std::fscanf(f, "m_Vec [ PINITMIN ].Set ( %f, %f, %f )\n ", &s.initmin[0], &s.initmin[1], &s.initmin[2]);
    ret += std::fscanf(f, "m_Vec [ PINITMAX ].Set ( %f, %f, %f )\n ", &s.initmax[0], &s.initmax[1], &s.initmax[2]);
    ret += std::fscanf(f, "m_Param [ PFORCE_MIN ] = %f\n ", &s.force_min);
    ret += std::fscanf(f, "m_Param [ PFORCE_FREQ ] = %f\n ", &s.force_freq);
    ret += std::fscanf(f, "m_Param [ PGROUND_SLOPE ] = %f\n ", &s.ground_slope);
    if (ret != 41) return bad("mg_read_simparams: " + std::to_string(ret) + " of 41 fields read from " + path);
    *sp = s;
    return MG_OK;
}

mg_status mg_write_simparams(const char* dir, const mg_simparams* s) {
    if (!dir || !s) return bad("mg_write_simparams: NULL argument");
    const std::string path = std::string(dir) + "/SimParams.txt";
    File fh(path.c_str(), "w");
    if (!fh.f) return bad("mg_write_simparams: cannot open " + path);
    const int ret = std::fprintf(
        fh.f,
        " m_Time = %f\n m_DT = %f\n m_Param [ PSIMSCALE ] = %f\n m_Param [ PGRID_DENSITY ] = %f\n"
        " m_Param [ PVISC ] = %f\n m_Param [ PSURFACE_TENSION ] = %f\n m_Param [ PRESTDENSITY ] = %f\n"
        " m_Param [ PSPACING ] = %f\n m_Param [ PMASS ] = %f\n m_Param [ PRADIUS ] = %f\n"
        " m_Param [ PDIST ] = %f\n m_Param [ PSMOOTHRADIUS ] = %f\n m_Param [ PINTSTIFF ] = %f\n"
        " m_Param [ PEXTSTIFF ] = %f\n m_Param [ PEXTDAMP ] = %f\n m_Param [ PACCEL_LIMIT ] = %f\n"
        " m_Param [ PVEL_LIMIT ] = %f\n m_Param [ PGRAV ] = %f\n m_Param [ PGROUND_SLOPE ] = %f\n"
        " m_Param [ PFORCE_MIN ] = %f\n m_Param [ PFORCE_MAX ] = %f\n m_Param [ PFORCE_FREQ ] = %f\n"
        " m_Vec [ PPLANE_GRAV_DIR ].Set ( %f, %f, %f )\n // Default sim config\n"
        " m_Param [ PGRIDSIZE ] = %f\n m_Vec [ PVOLMIN ].Set ( %f, %f, %f )\n"
        " m_Vec [ PVOLMAX ].Set ( %f, %f, %f )\n m_Vec [ PINITMIN ].Set ( %f, %f, %f )\n"
        " m_Vec [ PINITMAX ].Set ( %f, %f, %f )\n m_Param [ PFORCE_MIN ] = %f\n"
        " m_Param [ PFORCE_FREQ ] = %f\n m_Param [ PGROUND_SLOPE ] = %f\n ",
        s->time, s->dt, s->simscale, s->grid_density, s->visc, s->surface_tension, s->rest_density,
        s->spacing, s->mass, s->radius, s->dist, s->smooth_radius, s->intstiff, s->extstiff,
        s->extdamp, s->accel_limit, s->vel_limit, s->grav, s->ground_slope, s->force_min,
        s->force_max, s->force_freq, s->plane_grav_dir[0], s->plane_grav_dir[1],
        s->plane_grav_dir[2], s->grid_size, s->volmin[0], s->volmin[1], s->volmin[2], s->volmax[0],
        s->volmax[1], s->volmax[2], s->initmin[0], s->initmin[1], s->initmin[2], s->initmax[0],
        s->initmax[1], s->initmax[2], s->force_min, s->force_freq, s->ground_slope);
    if (ret < 0) return bad("mg_write_simparams: write failed for " + path);
    return MG_OK;
}

// ReadPointsCSV2's set-up of a simulation from SimParams (fileCL_IO.cpp:353-361): grid cell
// 2 * smooth radius / grid density, SetupSpacing's rest density / spacing relation and particle
// bounds, SetupGrid, and UpdateParams' gravity = plane gravity direction * gravity.
mg_status mg_fparams_from_simparams(const mg_simparams* s, int32_t gsrch_override, mg_fparams* p) {
    if (!s || !p) return bad("mg_fparams_from_simparams: NULL argument");
    if (!(s->simscale > 0.f) || !(s->grid_density > 0.f) || !(s->smooth_radius > 0.f))
        return bad("mg_fparams_from_simparams: simscale, grid density and smooth radius must be positive");
    mg_fparams q{};
    const float ss = s->simscale;
    const float grid_size = 2.f * s->smooth_radius / s->grid_density;
    float rest = s->rest_density;
    if (s->spacing != 0.f) {  // density from spacing (SetupSpacing)
        const float dist = s->spacing * ss / 0.87f;
        rest = s->mass / std::pow(dist, 3.0f);
    }
    q.psimscale = ss;
    q.psmoothradius = s->smooth_radius;
    q.pradius = s->radius;
    q.pmass = s->mass;
    q.prest_dens = rest;
    const double border = 2.0 * (grid_size / ss);
    for (int k = 0; k < 3; k++) {
        q.pboundmin[k] = (float)(s->volmin[k] + border);
        q.pboundmax[k] = (float)(s->volmax[k] - border);
        q.pgravity[k] = s->plane_grav_dir[k] * s->grav;
    }
    q.pextstiff = s->extstiff;
    q.pintstiff = s->intstiff;
    q.pvisc = s->visc;
    q.psurface_t = s->surface_tension;
    q.pdamp = s->extdamp;
    q.pforce_min = s->force_min;
    q.pforce_max = s->force_max;
    q.pforce_freq = s->force_freq;
    q.pground_slope = s->ground_slope;
    q.paccel_limit = s->accel_limit;
    q.pvel_limit = s->vel_limit;
    q.dt = s->dt;
    q.time = s->time;
    mg_status st = mg_setup_grid(&q, s->volmin, s->volmax, grid_size, gsrch_override);
    if (st != MG_OK) return st;
    *p = q;
    return MG_OK;
}

mg_status mg_read_genome(const char* path, mg_genome* out) {
    if (!path || !out) return bad("mg_read_genome: NULL argument");
    File fh(path, "rb");
    if (!fh.f) return bad(std::string("mg_read_genome: cannot open ") + path);
    FILE* f = fh.f;
    mg_genome g{};
    int ng = 0, ntf = 0;
    if (std::fscanf(f, "num genes = %i,\tnum transcription factors = %i \n", &ng, &ntf) != 2)
        return bad("mg_read_genome: header line not found");
    if (ng != MG_NUM_GENES || ntf != MG_NUM_TF)
        return bad("mg_read_genome: " + std::to_string(ng) + " genes / " + std::to_string(ntf) +
                   " transcription factors; this build has 16 / 16");
    skip(std::fscanf(f, "mutability, delay,\tsensitivity[NUM_GENES]"));
    for (int i = 0; i < MG_NUM_GENES; i++) skip(std::fscanf(f, ",\t"));
    skip(std::fscanf(f, "secrete[NUM_TF][2]"));
    for (int i = 0; i < MG_NUM_TF; i++) skip(std::fscanf(f, ",,\t"));
    skip(std::fscanf(f, "secrete[2*NUM_TF], "));
    skip(std::fscanf(f, "activate[NUM_GENES][2]"));
    for (int i = 0; i < MG_NUM_GENES; i++) skip(std::fscanf(f, ",,\t"));
    skip(std::fscanf(f, "activate[2*NUM_GENES]"));
    for (int i = 0; i < MG_NUM_GENES; i++) {
        int ret = std::fscanf(f, "%u,%u,", &g.mutability[i], &g.delay[i]);
        for (int j = 0; j < MG_NUM_TF; j++) ret += std::fscanf(f, "%f,", &g.sensitivity[i][j]);
        for (int j = 0; j < MG_NUM_TF; j++)
            ret += std::fscanf(f, "%f,%f,\t", &g.secrete[i][2 * j], &g.secrete[i][2 * j + 1]);
        ret += std::fscanf(f, "%f,\t\t", &g.secrete[i][2 * MG_NUM_TF]);
        for (int j = 0; j < MG_NUM_GENES; j++)
            ret += std::fscanf(f, "%f,%f,\t", &g.activate[i][2 * j], &g.activate[i][2 * j + 1]);
        ret += std::fscanf(f, "%f,\t\t \n", &g.activate[i][2 * MG_NUM_GENES]);
        if (ret != 2 + MG_NUM_TF + 2 * MG_NUM_TF + 1 + 2 * MG_NUM_GENES + 1)
            return bad("mg_read_genome: gene " + std::to_string(i) + ": " + std::to_string(ret) + " fields");
    }
    skip(std::fscanf(f, "\nTranscription Factors (tf_difusibility,tf_breakdown_rate) \n"));
    int ret = 0;
    for (int i = 0; i < MG_NUM_TF; i++) {
        ret += std::fscanf(f, "\t%f,\t", &g.tf_diffusability[i]);
        ret += std::fscanf(f, "%f,\t", &g.tf_breakdown_rate[i]);
    }
    if (ret != 2 * MG_NUM_TF) return bad("mg_read_genome: transcription factor rates");
    skip(std::fscanf(f, "\nRemodelling parameters, rows : elastin,collagen,apatite\n"));
    skip(std::fscanf(f, "\ncollumns : /*triggering bond parameter changes*/, /*triggering particle changes*/, /*initial values for new bonds*/"));
    skip(std::fscanf(f, "\nelongation_threshold,\telongation_factor,\tstrength_threshold,\tstrengthening_factor,\t\t"
                        "    max_rest_length,\tmin_rest_length,\tmax_modulus,\t\t\tmin_modulus,\t\t"
                        "    elastLim,\tdefault_rest_length,\tdefault_modulus,\tdefault_damping\n"));
    ret = 0;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 12; j++) ret += std::fscanf(f, "\t%f,\t", &g.param[i][j]);
        skip(std::fscanf(f, "\n"));
    }
    if (ret != 36) return bad("mg_read_genome: remodelling parameters");
    skip(std::fscanf(f, "\n\nBond remodelling m_FGenome.tanh_param[3][8] parameters, rows : elastin,collagen,apatite"));
    skip(std::fscanf(f, "\ncollumns : lengthen/shorten, strengthen/weaken"));
    skip(std::fscanf(f, "\nl_a (y-shift),\t l_b (y-scaling),\t l_c (x-scaling),\t l_d (x-shift),\t\t s_a (y-shift),"
                        "\t s_b (y-scaling),\t s_c (x-scaling),\t s_d (x-shift)\n"));
    ret = 0;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 8; j++) ret += std::fscanf(f, "\t%f,\t", &g.tanh_param[i][j]);
        skip(std::fscanf(f, "\n"));
    }
    if (ret != 24) return bad("mg_read_genome: tanh parameters");
    *out = g;
    return MG_OK;
}

mg_status mg_write_genome(const char* dir, const mg_genome* g, int32_t integer_fields) {
    if (!dir || !g) return bad("mg_write_genome: NULL argument");
    const std::string path = std::string(dir) + "/genome.csv";
    File fh(path.c_str(), "w");
    if (!fh.f) return bad("mg_write_genome: cannot open " + path);
    FILE* fp = fh.f;
    // the reference's fields are integers; with integer_fields the floats are rounded
    auto num = [&](float v, const char* sep) {
        if (integer_fields) std::fprintf(fp, "%i%s", (int)std::lround(v), sep);
        else std::fprintf(fp, "%.9g%s", v, sep);
    };
    std::fprintf(fp, "num genes = %i,\tnum transcription factors = %i \n", MG_NUM_GENES, MG_NUM_TF);
    std::fprintf(fp, "mutability, delay,\tsensitivity[NUM_GENES]");
    for (int i = 0; i < MG_NUM_GENES; i++) std::fprintf(fp, ",\t");
    std::fprintf(fp, "secrete[NUM_TF][2]");
    for (int i = 0; i < MG_NUM_TF; i++) std::fprintf(fp, ",,\t");
    std::fprintf(fp, "secrete[2*NUM_TF], ");
    std::fprintf(fp, "activate[NUM_GENES][2]");
    for (int i = 0; i < MG_NUM_GENES; i++) std::fprintf(fp, ",,\t");
    std::fprintf(fp, "activate[2*NUM_GENES] \n");
    for (int i = 0; i < MG_NUM_GENES; i++) {
        std::fprintf(fp, "%u,\t", g->mutability[i]);
        std::fprintf(fp, "%u,\t\t", g->delay[i]);
        for (int j = 0; j < MG_NUM_TF; j++) num(g->sensitivity[i][j], ",\t");
        std::fprintf(fp, " \t\t");
        for (int j = 0; j < MG_NUM_TF; j++) {
            num(g->secrete[i][2 * j], ",");
            num(g->secrete[i][2 * j + 1], ",\t");
        }
        std::fprintf(fp, "\t\t");
        num(g->secrete[i][2 * MG_NUM_TF], ",\t\t");
        for (int j = 0; j < MG_NUM_GENES; j++) {
            num(g->activate[i][2 * j], ",");
            num(g->activate[i][2 * j + 1], ",\t");
        }
        std::fprintf(fp, "\t\t");
        num(g->activate[i][2 * MG_NUM_GENES], ",\t\t");
        std::fprintf(fp, " \n");
    }
    std::fprintf(fp, "\nTranscription Factors (tf_difusibility,tf_breakdown_rate) \n");
    for (int i = 0; i < MG_NUM_TF; i++) {
        std::fprintf(fp, "\t");
        num(g->tf_diffusability[i], ",\t");
        num(g->tf_breakdown_rate[i], ",\t");
    }
    std::fprintf(fp, "\n\nRemodelling parameters, rows : elastin,collagen,apatite");
    std::fprintf(fp, "\ncollumns : /*triggering bond parameter changes*/, /*triggering particle changes*/, /*initial values for new bonds*/");
    std::fprintf(fp, "\nelongation_threshold,\telongation_factor,\tstrength_threshold,\tstrengthening_factor,\t\t"
                     "    max_rest_length,\tmin_rest_length,\tmax_modulus,\t\t\tmin_modulus,\t\t"
                     "    elastLim,\tdefault_rest_length,\tdefault_modulus,\tdefault_damping\n");
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 12; j++) std::fprintf(fp, "\t%f,\t", g->param[i][j]);
        std::fprintf(fp, "\n");
    }
    std::fprintf(fp, "\n\nBond remodelling m_FGenome.tanh_param[3][8] parameters, rows : elastin,collagen,apatite");
    std::fprintf(fp, "\ncollumns : lengthen/shorten, strengthen/weaken");
    std::fprintf(fp, "\nl_a (y-shift),\t l_b (y-scaling),\t l_c (x-scaling),\t l_d (x-shift),\t\t s_a (y-shift),"
                     "\t s_b (y-scaling),\t s_c (x-scaling),\t s_d (x-shift)\n");
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 8; j++) std::fprintf(fp, "\t%f,\t", g->tanh_param[i][j]);
        std::fprintf(fp, "\n");
    }
    return MG_OK;
}

mg_status mg_count_points_csv(const char* path, uint32_t* n) {
    if (!path || !n) return bad("mg_count_points_csv: NULL argument");
    File fh(path, "rb");
    if (!fh.f) return bad(std::string("mg_count_points_csv: cannot open ") + path);
    uint64_t lines = 0;
    int ch;
    while ((ch = std::getc(fh.f)) != EOF)
        if (ch == '\n') ++lines;
    if (lines == 0) return bad("mg_count_points_csv: empty file");
    *n = (uint32_t)(lines - 1);  // one header line (ReadPointsCSV2)
    return MG_OK;
}

// index of (particle i, species j) in the points' conc array
static size_t conc_at(const mg_points* p, uint32_t i, int j) {
    return p->conc_species_major ? (size_t)j * p->n + i : (size_t)i * MG_NUM_TF + j;
}

static bool points_ok(const mg_points* p) {
    return p && p->pos && p->vel && p->age && p->color && p->elastidx && p->particle_id &&
           p->mass_radius && p->nerve && p->pidx && p->conc && p->epigen;
}

mg_status mg_write_points_csv(const char* dir, int32_t frame, const mg_points* p) {
    if (!dir || !points_ok(p)) return bad("mg_write_points_csv: NULL argument");
    char buf[1024];
    std::snprintf(buf, sizeof buf, "%s/particles_pos_vel_color%04d.csv", dir, frame + 100000);
    File fh(buf, "w");
    if (!fh.f) return bad(std::string("mg_write_points_csv: cannot open ") + buf);
    FILE* fp = fh.f;
    const uint32_t n = p->n;
    std::fprintf(fp, "i,, x coord, y coord, z coord\t\t x vel, y vel, z vel\t\t age,  color\t\t FELASTIDX[%u*%u]",
                 (unsigned)MG_BONDS_PER_PARTICLE, (unsigned)MG_DATA_PER_BOND);
    for (int i = 0; i < MG_BONDS_PER_PARTICLE; i++)
        std::fprintf(fp, ",(%u)[0]curIdx, [1]elastLim, [2]restLn, [3]modulus, [4]damping, [5]partID, "
                         "[6]stress_sq integrator, [7]stress integrator, [8]change-type,,  ", (unsigned)i);
    std::fprintf(fp, "\t");
    std::fprintf(fp, "\tParticle_ID, mass, radius, FNERVEIDX,\t\t Particle_Idx[%u*2]", (unsigned)MG_BONDS_PER_PARTICLE);
    for (int i = 0; i < MG_BONDS_PER_PARTICLE; i++) std::fprintf(fp, "%u,,, ", (unsigned)i);
    std::fprintf(fp, "\t\tFCONC[%u] ", (unsigned)MG_NUM_TF);
    for (int i = 0; i < MG_NUM_TF; i++) std::fprintf(fp, "%u, ", (unsigned)i);
    std::fprintf(fp, "\t\tFEPIGEN[%u] ", (unsigned)MG_NUM_GENES);
    for (int i = 0; i < MG_NUM_GENES; i++) std::fprintf(fp, "%u, ", (unsigned)i);
    std::fprintf(fp, "\n");
    for (uint32_t i = 0; i < n; i++) {
        const float* ps = p->pos + 4 * (size_t)i;
        const float* vl = p->vel + 4 * (size_t)i;
        std::fprintf(fp, "%u,,%f,%f,%f,\t%f,%f,%f,\t %u, %u,, \t", i, ps[0], ps[1], ps[2], vl[0], vl[1], vl[2],
                     p->age[i], p->color[i]);
        const uint32_t* eu = p->elastidx + (size_t)i * MG_BOND_DATA;
        float ef[MG_BOND_DATA];
        std::memcpy(ef, eu, sizeof ef);
        for (int j = 0; j < MG_BOND_DATA; j += MG_DATA_PER_BOND) {
            std::fprintf(fp, "%u, %f, %f, %f, %f, %u, %f, %f, %u, ", eu[j], ef[j + 1], ef[j + 2], ef[j + 3],
                         ef[j + 4], eu[j + 5], ef[j + 6], ef[j + 7], eu[j + 8]);
            std::fprintf(fp, "\t\t");
        }
        const uint32_t mr = p->mass_radius[i];
        std::fprintf(fp, " \t%u, %u, %u, %u, \t\t", p->particle_id[i], mr & 0xFFFFu, mr >> 16, p->nerve[i]);
        const uint32_t* pi = p->pidx + (size_t)i * 2 * MG_BONDS_PER_PARTICLE;
        for (int j = 0; j < 2 * MG_BONDS_PER_PARTICLE; j += 2) std::fprintf(fp, "%u, %u,, ", pi[j], pi[j + 1]);
        std::fprintf(fp, "\t\t");
        for (int j = 0; j < MG_NUM_TF; j++) std::fprintf(fp, "%f, ", p->conc[conc_at(p, i, j)]);
        std::fprintf(fp, "\t\t");
        for (int j = 0; j < MG_NUM_GENES; j++) std::fprintf(fp, "%u, ", p->epigen[(size_t)j * n + i]);
        std::fprintf(fp, " \n");
    }
    return MG_OK;
}

mg_status mg_read_points_csv(const char* path, mg_points* p) {
    if (!path || !points_ok(p)) return bad("mg_read_points_csv: NULL argument");
    File fh(path, "rb");
    if (!fh.f) return bad(std::string("mg_read_points_csv: cannot open ") + path);
    FILE* f = fh.f;
    unsigned bonds = 0, per_bond = 0, bpp = 0, ntf = 0, ngenes = 0, discard = 0;
    if (std::fscanf(f, "i,, x coord, y coord, z coord\t\t x vel, y vel, z vel\t\t age,  color\t\t FELASTIDX[%u*%u]",
                    &bonds, &per_bond) != 2)
        return bad("mg_read_points_csv: header not found");
    for (unsigned i = 0; i < bonds; i++)
        skip(std::fscanf(f, ",(%u)[0]curIdx, [1]elastLim, [2]restLn, [3]modulus, [4]damping, [5]partID, "
                            "[6]stress_sq integrator, [7]stress integrator, [8]change-type,,  ", &discard));
    skip(std::fscanf(f, "\t"));
    skip(std::fscanf(f, "\tParticle_ID, mass, radius, FNERVEIDX,\t\t Particle_Idx[%u*2]", &bpp));
    for (unsigned i = 0; i < bpp; i++) skip(std::fscanf(f, "%u,,, ", &discard));
    skip(std::fscanf(f, "\t\tFCONC[%u]", &ntf));
    for (unsigned i = 0; i < ntf; i++) skip(std::fscanf(f, "%u, ", &discard));
    skip(std::fscanf(f, "\t\tFEPIGEN[%u] ", &ngenes));
    for (unsigned i = 0; i < ngenes; i++) skip(std::fscanf(f, "%u, ", &discard));
    skip(std::fscanf(f, "\n"));
    if (bonds != MG_BONDS_PER_PARTICLE || per_bond != MG_DATA_PER_BOND || bpp != MG_BONDS_PER_PARTICLE ||
        ntf != MG_NUM_TF || ngenes != MG_NUM_GENES)
        return bad("mg_read_points_csv: the file's bond/species/gene counts differ from 6/9/16/16");
    const uint32_t n = p->n;
    for (uint32_t i = 0; i < n; i++) {
        unsigned index = 0, age = 0, clr = 0;
        float ps[3], vl[3];
        int ret = std::fscanf(f, "%u,,%f,%f,%f,\t%f,%f,%f,\t %u, %u,, \t", &index, &ps[0], &ps[1], &ps[2],
                              &vl[0], &vl[1], &vl[2], &age, &clr);
        uint32_t* eu = p->elastidx + (size_t)i * MG_BOND_DATA;
        for (int j = 0; j < MG_BOND_DATA; j += MG_DATA_PER_BOND) {
            float a1, a2, a3, a4, a6, a7;
            unsigned u0, u5, u8;
            ret += std::fscanf(f, "%u, %f, %f, %f, %f, %u, %f, %f, %u, ", &u0, &a1, &a2, &a3, &a4, &u5, &a6, &a7, &u8);
            eu[j] = u0;
            std::memcpy(&eu[j + 1], &a1, 4);
            std::memcpy(&eu[j + 2], &a2, 4);
            std::memcpy(&eu[j + 3], &a3, 4);
            std::memcpy(&eu[j + 4], &a4, 4);
            eu[j + 5] = u5;
            std::memcpy(&eu[j + 6], &a6, 4);
            std::memcpy(&eu[j + 7], &a7, 4);
            eu[j + 8] = u8;
        }
        unsigned id = 0, mass = 0, radius = 0, nerve = 0;
        ret += std::fscanf(f, " \t%u, %u, %u, %u, \t\t", &id, &mass, &radius, &nerve);
        uint32_t* pi = p->pidx + (size_t)i * 2 * MG_BONDS_PER_PARTICLE;
        for (int j = 0; j < 2 * MG_BONDS_PER_PARTICLE; j += 2) ret += std::fscanf(f, "%u, %u,, ", &pi[j], &pi[j + 1]);
        for (int j = 0; j < MG_NUM_TF; j++) ret += std::fscanf(f, "%f, ", &p->conc[conc_at(p, i, j)]);
        skip(std::fscanf(f, "\t"));
        for (int j = 0; j < MG_NUM_GENES; j++) ret += std::fscanf(f, "%u, ", &p->epigen[(size_t)j * n + i]);
        skip(std::fscanf(f, " \n"));
        if (ret != 9 + MG_BOND_DATA + 4 + 2 * MG_BONDS_PER_PARTICLE + MG_NUM_TF + MG_NUM_GENES)
            return bad("mg_read_points_csv: particle line " + std::to_string(i + 1) + ": " + std::to_string(ret) +
                       " of 111 fields");
        float* po = p->pos + 4 * (size_t)i;
        float* vo = p->vel + 4 * (size_t)i;
        po[0] = ps[0]; po[1] = ps[1]; po[2] = ps[2]; po[3] = 0.f;
        vo[0] = vl[0]; vo[1] = vl[1]; vo[2] = vl[2]; vo[3] = 0.f;
        p->age[i] = age;
        p->color[i] = clr;
        p->particle_id[i] = id;
        p->mass_radius[i] = mass + (radius << 16);  // two 16-bit halves (ReadPointsCSV2)
        p->nerve[i] = nerve;
    }
    return MG_OK;
}

// ---- SpecificationFile.txt (ReadSpecificationFile fileCL_IO.cpp:742-879,
//      WriteSpecificationFile_fromLaunchParams :1006-1114) ----------------------------------
mg_status mg_read_specification(const char* dir, mg_spec* out) {
    if (!dir || !out) return bad("mg_read_specification: NULL argument");
    const std::string path = std::string(dir) + "/SpecificationFile.txt";
    File fh(path.c_str(), "rb");
    if (!fh.f) return bad("mg_read_specification: cannot open " + path);
    FILE* f = fh.f;
    mg_spec s{};
    int ret = 0;
    ret += std::fscanf(f, "num_particles = %u\n ", &s.num_particles);
    ret += std::fscanf(f, "demoType = %u\n ", &s.demo_type);
    ret += std::fscanf(f, "simSpace = %u\n ", &s.sim_space);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "m_Time = %f\n ", &s.time);
    ret += std::fscanf(f, "m_DT = %f\n ", &s.dt);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "gridsize = %f\n ", &s.gridsize);
    ret += std::fscanf(f, "spacing = %f\n ", &s.spacing);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "simscale = %f\n ", &s.simscale);
    ret += std::fscanf(f, "smooth_radius = %f\n ", &s.smooth_radius);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "visc = %f\n ", &s.visc);
    ret += std::fscanf(f, "surface_t = %f\n ", &s.surface_tension);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "mass = %f\n ", &s.mass);
    ret += std::fscanf(f, "radius = %f\n ", &s.radius);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "int_stiff = %f\n ", &s.intstiff);
    ret += std::fscanf(f, "ext_stiff = %f\n ", &s.extstiff);
    ret += std::fscanf(f, "ext_damp = %f\n ", &s.extdamp);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "accel_limit = %f\n ", &s.accel_limit);
    ret += std::fscanf(f, "vel_limit = %f\n ", &s.vel_limit);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "grav = %f\n ", &s.grav);
    ret += std::fscanf(f, "slope = %f\n ", &s.ground_slope);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "force_min = %f\n ", &s.force_min);
    ret += std::fscanf(f, "force_max = %f\n ", &s.force_max);
    ret += std::fscanf(f, "force_freq = %f\n ", &s.force_freq);
    skip(std::fscanf(f, "\n"));
    static const char* const vec_names[6] = {"%s_dim", "pos_%s", "volmin_%s", "volmax_%s", "initmin_%s", "initmax_%s"};
    float* vecs[6] = {s.dim, s.pos, s.volmin, s.volmax, s.initmin, s.initmax};
    static const char* const axis[3] = {"x", "y", "z"};
    for (int v = 0; v < 6; v++) {
        for (int k = 0; k < 3; k++) {
            char name[32], fmt[64];
            std::snprintf(name, sizeof name, vec_names[v], axis[k]);
            std::snprintf(fmt, sizeof fmt, "%s = %%f\n ", name);
            ret += std::fscanf(f, fmt, &vecs[v][k]);
        }
        skip(std::fscanf(f, "\n"));
    }
    ret += std::fscanf(f, "paramsPath = %255s\n ", s.params_path);
    ret += std::fscanf(f, "pointsPath = %255s\n ", s.points_path);
    ret += std::fscanf(f, "genomePath = %255s\n ", s.genome_path);
    ret += std::fscanf(f, "outPath = %255s\n ", s.out_path);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "num_files = %u\n ", &s.num_files);
    ret += std::fscanf(f, "steps_per_InnerPhysicalLoop = %u\n ", &s.steps_per_inner_loop);
    ret += std::fscanf(f, "steps_per_file = %u\n ", &s.steps_per_file);
    ret += std::fscanf(f, "freeze_steps = %u\n ", &s.freeze_steps);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "debug = %u\n ", &s.debug);
    ret += std::fscanf(f, "file_num = %u\n ", &s.file_num);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "save_ply = %c\n ", &s.save_ply);
    ret += std::fscanf(f, "save_csv = %c\n ", &s.save_csv);
    ret += std::fscanf(f, "save_vtp = %c\n ", &s.save_vtp);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "gene_activity = %c\n ", &s.gene_activity);
    ret += std::fscanf(f, "remodelling = %c\n ", &s.remodelling);
    ret += std::fscanf(f, "read_genome = %c\n ", &s.read_genome);
    skip(std::fscanf(f, "\n"));
    ret += std::fscanf(f, "actuation_factor = %f\n ", &s.actuation_factor);
    ret += std::fscanf(f, "actuation_period = %f\n ", &s.actuation_period);
    if (ret != 59) return bad("mg_read_specification: " + std::to_string(ret) + " of 59 fields read from " + path);
    *out = s;
    return MG_OK;
}

mg_status mg_write_specification(const char* dir, const mg_spec* s) {
    if (!dir || !s) return bad("mg_write_specification: NULL argument");
    for (const char* p : {s->params_path, s->points_path, s->genome_path, s->out_path})
        if (std::memchr(p, 0, 256) == nullptr) return bad("mg_write_specification: a path is not terminated");
    const std::string path = std::string(dir) + "/SpecificationFile.txt";
    File fh(path.c_str(), "w");
    if (!fh.f) return bad("mg_write_specification: cannot open " + path);
    FILE* f = fh.f;
    int ret = 0;
    auto chk = [&](int r) { if (r < 0) ret = -1; };
    chk(std::fprintf(f, "num_particles = %u\n demoType = %u\n simSpace = %u\n \n", s->num_particles, s->demo_type, s->sim_space));
    chk(std::fprintf(f, "m_Time = %f\n m_DT = %f\n \n", s->time, s->dt));
    chk(std::fprintf(f, "gridsize = %f\n spacing = %f\n \n", s->gridsize, s->spacing));
    chk(std::fprintf(f, "simscale = %f\n smooth_radius = %f\n \n", s->simscale, s->smooth_radius));
    chk(std::fprintf(f, "visc = %f\n surface_t = %f\n \n", s->visc, s->surface_tension));
    chk(std::fprintf(f, "mass = %f\n radius = %f\n \n", s->mass, s->radius));
    chk(std::fprintf(f, "int_stiff = %f\n ext_stiff = %f\n ext_damp = %f\n \n", s->intstiff, s->extstiff, s->extdamp));
    chk(std::fprintf(f, "accel_limit = %f\n vel_limit = %f\n \n", s->accel_limit, s->vel_limit));
    chk(std::fprintf(f, "grav = %f\n slope = %f\n \n", s->grav, s->ground_slope));
    chk(std::fprintf(f, "force_min = %f\n force_max = %f\n force_freq = %f\n \n", s->force_min, s->force_max, s->force_freq));
    chk(std::fprintf(f, "x_dim = %f\n y_dim = %f\n z_dim = %f\n \n", s->dim[0], s->dim[1], s->dim[2]));
    chk(std::fprintf(f, "pos_x = %f\n pos_y = %f\n pos_z = %f\n \n", s->pos[0], s->pos[1], s->pos[2]));
    const char* const names[4] = {"volmin", "volmax", "initmin", "initmax"};
    const float* const vecs[4] = {s->volmin, s->volmax, s->initmin, s->initmax};
    for (int v = 0; v < 4; v++)
        chk(std::fprintf(f, "%s_x = %f\n %s_y = %f\n %s_z = %f\n \n", names[v], vecs[v][0], names[v], vecs[v][1],
                         names[v], vecs[v][2]));
    chk(std::fprintf(f, "paramsPath = %s\n pointsPath = %s\n genomePath = %s\n outPath = %s\n \n", s->params_path,
                     s->points_path, s->genome_path, s->out_path));
    chk(std::fprintf(f, "num_files = %u\n steps_per_InnerPhysicalLoop = %u\n steps_per_file = %u\n freeze_steps = %u\n \n",
                     s->num_files, s->steps_per_inner_loop, s->steps_per_file, s->freeze_steps));
    chk(std::fprintf(f, "debug = %u\n file_num = %u\n \n", s->debug, s->file_num));
    chk(std::fprintf(f, "save_ply = %c\n save_csv = %c\n save_vtp = %c\n \n", s->save_ply, s->save_csv, s->save_vtp));
    chk(std::fprintf(f, "gene_activity = %c\n remodelling = %c\n read_genome = %c\n \n", s->gene_activity,
                     s->remodelling, s->read_genome));
    chk(std::fprintf(f, "actuation_factor = %f\n actuation_period = %f\n \n", s->actuation_factor, s->actuation_period));
    if (ret < 0) return bad("mg_write_specification: write failed for " + path);
    return MG_OK;
}

// ---- results.csv (WriteResultsCSV, fileCL_IO.cpp:1117-1142) ----------------------------------
mg_status mg_write_results_csv(const char* input_folder, const char* output_folder, const mg_spec* spec,
                               uint32_t num_particles_start, uint32_t num_particles_end,
                               uint32_t num_bonds_start, const uint32_t* elastidx, uint32_t n) {
    if (!input_folder || !output_folder || !spec || (!elastidx && n)) return bad("mg_write_results_csv: NULL argument");
    uint32_t bonds = 0;
    for (size_t k = 0; k < (size_t)n * MG_BONDS_PER_PARTICLE; k++) {
        float rest;
        std::memcpy(&rest, &elastidx[k * MG_DATA_PER_BOND + 2], 4);
        if (rest > 0.f) bonds++;
    }
    const uint32_t timesteps = (spec->num_files / 100) * spec->steps_per_inner_loop * spec->steps_per_file;
    const std::string path = std::string(output_folder) + "/results.csv";
    File fh(path.c_str(), "w");
    if (!fh.f) return bad("mg_write_results_csv: cannot open " + path);
    const int r = std::fprintf(fh.f,
                               "input_folder=,%s,\toutput_folder=,%s,\tfreeze_steps=,%u,\ttimesteps=,%u,\t"
                               "num_particles_start=,%u,\tnum_particles_end=,%u,\tnum_bonds_start=,%u,\t"
                               "num_bonds_end=,%u,\t\n",
                               input_folder, output_folder, spec->freeze_steps, timesteps, num_particles_start,
                               num_particles_end, num_bonds_start, bonds);
    if (r < 0) return bad("mg_write_results_csv: write failed for " + path);
    return MG_OK;
}

}  // extern "C"

// ---- VTP frames (SavePointsVTP2, fileCL_IO.cpp:1223-1655), VTK XML PolyData in ASCII ----------
namespace {
struct Xml {
    FILE* f;
    bool ok = true;
    void put(const char* s) { ok &= std::fputs(s, f) >= 0; }
    template <class... T> void fmt(const char* s, T... v) { ok &= std::fprintf(f, s, v...) >= 0; }
    void open_array(const char* type, const char* name, int comps) {
        fmt("        <DataArray type=\"%s\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"ascii\">\n", type, name,
            comps);
    }
    void close_array() { put("\n        </DataArray>\n"); }
};
}  // namespace

extern "C" {

mg_status mg_write_points_vtp(const char* dir, int32_t frame, const mg_points* p, uint32_t active,
                              const float* veval, const float* force, const float* press, const float* invdens,
                              const float volmin[3], const float volmax[3]) {
    if (!dir || !points_ok(p) || !veval || !force || !press || !invdens || !volmin || !volmax)
        return bad("mg_write_points_vtp: NULL argument");
    if (active > p->n) return bad("mg_write_points_vtp: active exceeds the particle count");
    char buf[1024];
    std::snprintf(buf, sizeof buf, "%s/particles_pos_vel_color%04d.vtp", dir, frame + 100000);
    File fh(buf, "w");
    if (!fh.f) return bad(std::string("mg_write_points_vtp: cannot open ") + buf);
    Xml x{fh.f};
    const uint32_t n = p->n, np = active + 8, B = MG_BONDS_PER_PARTICLE;
    const uint64_t nlines = (uint64_t)np * B;
    auto bond_word = [&](uint32_t i, int b, int w) { return p->elastidx[(size_t)i * MG_BOND_DATA + b * MG_DATA_PER_BOND + w]; };
    auto bond_float = [&](uint32_t i, int b, int w) {
        float v;
        const uint32_t u = bond_word(i, b, w);
        std::memcpy(&v, &u, 4);
        return v;
    };
    x.put("<?xml version=\"1.0\"?>\n<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
          "  <PolyData>\n");
    x.fmt("    <Piece NumberOfPoints=\"%u\" NumberOfVerts=\"0\" NumberOfLines=\"%llu\" NumberOfStrips=\"0\" "
          "NumberOfPolys=\"0\">\n", np, (unsigned long long)nlines);
    // point data: particles, then the 8 corners with zeros
    x.put("      <PointData>\n");
    auto u32_points = [&](const char* name, const uint32_t* a) {
        x.open_array("UInt32", name, 1);
        for (uint32_t i = 0; i < active; i++) x.fmt("%u ", a[i]);
        for (int c = 0; c < 8; c++) x.put("0 ");
        x.close_array();
    };
    u32_points("FAGE", p->age);
    u32_points("FCLR", p->color);
    u32_points("FPARTICLE_ID", p->particle_id);
    x.open_array("UInt32", "FMASS_RADIUS", 2);
    for (uint32_t i = 0; i < active; i++) x.fmt("%u %u ", p->mass_radius[i] & 0xFFFFu, p->mass_radius[i] >> 16);
    for (int c = 0; c < 8; c++) x.put("0 0 ");
    x.close_array();
    u32_points("FNERVEIDX", p->nerve);
    auto vec_points = [&](const char* name, const float* a) {
        x.open_array("Float32", name, 3);
        for (uint32_t i = 0; i < active; i++) x.fmt("%.9g %.9g %.9g ", a[4 * i], a[4 * i + 1], a[4 * i + 2]);
        for (int c = 0; c < 8; c++) x.put("0 0 0 ");
        x.close_array();
    };
    vec_points("FVEL", p->vel);
    vec_points("FVEVAL", veval);
    vec_points("FFORCE", force);
    x.open_array("Float32", "FPRESS", 1);
    for (uint32_t i = 0; i < active; i++) x.fmt("%.9g ", press[i]);
    for (int c = 0; c < 8; c++) x.put("0 ");
    x.close_array();
    x.open_array("Float32", "FDENSITY,(1/density,density)", 2);
    for (uint32_t i = 0; i < active; i++) x.fmt("%.9g %.9g ", invdens[i], invdens[i] == 0.f ? 0.f : 1.f / invdens[i]);
    for (int c = 0; c < 8; c++) x.put("0 0 ");
    x.close_array();
    for (int t = 0; t < MG_NUM_TF; t++) {
        char name[32];
        std::snprintf(name, sizeof name, "FCONC_%d", t);
        x.open_array("Float32", name, 1);
        for (uint32_t i = 0; i < active; i++) x.fmt("%.9g ", p->conc[conc_at(p, i, t)]);
        for (int c = 0; c < 8; c++) x.put("0 ");
        x.close_array();
    }
    for (int g = 0; g < MG_NUM_GENES; g++) {
        char name[32];
        std::snprintf(name, sizeof name, "FEPIGEN_%d", g);
        u32_points(name, p->epigen + (size_t)g * n);
    }
    x.open_array("UInt32", "F_TISSUE_TYPE", 1);
    for (uint32_t i = 0; i < active; i++) {
        auto on = [&](int g) { return p->epigen[(size_t)g * n + i] > 0u; };
        const unsigned t = on(9) ? 9 : on(6) ? 6 : on(7) ? 7 : on(10) ? 10 : on(8) ? 8 : 0;
        x.fmt("%u ", t);
    }
    for (int c = 0; c < 8; c++) x.put("0 ");
    x.close_array();
    x.put("      </PointData>\n      <CellData>\n");
    // cell data: one tuple per line (bond slot); the corners' lines carry zeros
    x.open_array("UInt32", "parent_idx, parent_ID, curr_idx, particle ID, bond index", 6);
    for (uint32_t i = 0; i < active; i++)
        for (int b = 0; b < (int)B; b++)
            x.fmt("%u %u %u %u %d 0 ", i, p->particle_id[i], bond_word(i, b, 0), bond_word(i, b, 5), b);
    for (uint32_t c = 0; c < 8 * B; c++) x.put("0 0 0 0 0 0 ");
    x.close_array();
    static const char* const fnames[6] = {"elastic_limit", "restlength", "modulus", "damping_coeff",
                                          "strain_integrator", "strain_sq_integrator"};
    static const int fwords[6] = {1, 2, 3, 4, 7, 6};
    for (int a = 0; a < 6; a++) {
        x.open_array("Float32", fnames[a], 1);
        for (uint32_t i = 0; i < active; i++)
            for (int b = 0; b < (int)B; b++) x.fmt("%.9g ", bond_float(i, b, fwords[a]));
        for (uint32_t c = 0; c < 8 * B; c++) x.put("0 ");
        x.close_array();
    }
    x.put("      </CellData>\n      <Points>\n");
    x.open_array("Float32", "Points", 3);
    for (uint32_t i = 0; i < active; i++) x.fmt("%.9g %.9g %.9g ", p->pos[4 * i], p->pos[4 * i + 1], p->pos[4 * i + 2]);
    for (int c = 0; c < 8; c++)
        x.fmt("%.9g %.9g %.9g ", (c & 1) ? volmax[0] : volmin[0], (c & 2) ? volmax[1] : volmin[1],
              (c & 4) ? volmax[2] : volmin[2]);
    x.close_array();
    x.put("      </Points>\n      <Lines>\n");
    x.put("        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n");
    for (uint32_t i = 0; i < np; i++)
        for (int b = 0; b < (int)B; b++) {
            uint32_t j = i;
            if (i < active) {
                const uint32_t partner = bond_word(i, b, 0);
                if (!(bond_float(i, b, 2) < 0.000001f) && partner < active) j = partner;
            }
            x.fmt("%u %u ", i, j);
        }
    x.close_array();
    x.put("        <DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n");
    for (uint64_t l = 1; l <= nlines; l++) x.fmt("%llu ", (unsigned long long)(2 * l));
    x.close_array();
    x.put("      </Lines>\n    </Piece>\n  </PolyData>\n</VTKFile>\n");
    if (!x.ok) return bad(std::string("mg_write_points_vtp: write failed for ") + buf);
    return MG_OK;
}

}  // extern "C"
