// mg_files.cpp - the reference's text file formats: SimParams.txt, genome.csv and the particle
// CSV written by SavePointsCSV2, with the parameter set-up ReadPointsCSV2 performs.
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

}  // extern "C"
