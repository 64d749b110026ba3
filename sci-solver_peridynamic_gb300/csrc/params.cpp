// params.cpp -- the parameter surface of the reference (SystemParameter).
//
//   pd_params_default   SystemParameter::initParameters   src/core/parameters.cu:40-86
//                       RunningParameters()               src/core/parameters.h:92-104
//   pd_params_load      loadParametersFromFile            src/core/parameters.cu:89-347
//   pd_params_derive    calculateDependentParameters      src/core/parameters.cu:351-453
// Keys, defaults and derived quantities follow the reference exactly,
// including its float-typed fmaxf() for the cell size and the float fields
// of RunningParameters.  SPH-only keys are accepted and ignored.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "pd_gb300.h"

namespace {

constexpr double kPi = 3.14159265358979323846264;        // definitions.h:63 (PI)
constexpr double kMinDistance = 0.0005;                   // definitions.h:84 (PERIDYNAMICS_MIN_DISTANCE)
constexpr int kNumCellX = 32, kNumCellY = 32, kNumCellZ = 64;   // definitions.h:54-56
constexpr int kTimestepPD = 128;                          // definitions.h:68

}  // namespace

extern "C" pd_status pd_params_default(pd_sim_params* s, pd_run_params* r)
{
    if (!s || !r) return PD_ERR_INVALID_ARGUMENT;
    std::memset(s, 0, sizeof(*s));
    std::memset(r, 0, sizeof(*r));
    s->num_pd_particle = 0;
    s->num_cell_x = s->num_cell_y = s->num_cell_z = 1;
    s->num_cells = 1;
    s->sph_kernel_coeff = 4.001f;           // float literal in the reference
    s->pd_kernel_coeff = 6.001;
    s->sph_particle_mass = 1.0f;
    s->pd_particle_mass = 1.0f;
    s->boundary_min_x = s->boundary_min_y = s->boundary_min_z = 0.0f;
    s->boundary_max_x = s->boundary_max_y = s->boundary_max_z = 1.0f;
    s->sph_particle_radius = 0.0f;
    s->pd_particle_radius = 0.0f;
    s->pd_horizon = 0.0f;
    s->pd_C_times_V = 0.0f;
    s->clockScale = 0.0f;
    r->gpu_device = 0;
    r->step_per_frame = 1;
    r->final_step = 1;
    r->dump_density = 0;
    r->dump_velocity = 0;
    r->wall_thickness = 20;
    r->mesh_translation_x = r->mesh_translation_y = r->mesh_translation_z = 0.0f;
    r->sph_initial_velocity = 1.0f;
    r->integrator = PD_IMPLICIT_EULER;
    return PD_OK;
}

extern "C" pd_status pd_params_derive(pd_sim_params* s, pd_run_params* r)
{
    if (!s || !r) return PD_ERR_INVALID_ARGUMENT;
    s->num_cell_x = kNumCellX;
    s->num_cell_y = kNumCellY;
    s->num_cell_z = kNumCellZ;
    s->num_cells = kNumCellX * kNumCellY * kNumCellZ;
    // fmaxf of the reference takes floats (parameters.cu:360-363)
    const float a = (float)((s->boundary_max_x - s->boundary_min_x) / kNumCellX);
    const float b = (float)((s->boundary_max_y - s->boundary_min_y) / kNumCellY);
    const float c = (float)((s->boundary_max_z - s->boundary_min_z) / kNumCellZ);
    const float ab = a > b ? a : b;
    s->cell_size = (double)(ab > c ? ab : c);
    const double smooth = s->cell_size;
    s->sph_particle_radius = s->cell_size / s->sph_kernel_coeff;
    s->pd_time_step = kTimestepPD;
    s->pd_particle_radius *= s->sph_particle_radius;
    s->pd_horizon = s->pd_particle_radius * s->pd_kernel_coeff;
    s->pd_C_times_V = (18.0 / kPi / 2.0 / 1296.0 / s->pd_particle_radius);
    s->scaleFactor = 2 * s->pd_particle_radius / kMinDistance;
    s->boundary_min_x /= s->scaleFactor;
    s->boundary_max_x /= s->scaleFactor;
    s->boundary_min_y /= s->scaleFactor;
    s->boundary_max_y /= s->scaleFactor;
    s->boundary_min_z /= s->scaleFactor;
    s->boundary_max_z /= s->scaleFactor;
    s->sph_particle_radius /= s->scaleFactor;
    s->pd_particle_radius /= s->scaleFactor;
    s->cell_size /= s->scaleFactor;
    s->pd_horizon /= s->scaleFactor;
    (void)smooth;
    (void)r;
    return PD_OK;
}

extern "C" pd_status pd_params_load(const char* path, pd_sim_params* s, pd_run_params* r)
{
    if (!path || !s || !r) return PD_ERR_INVALID_ARGUMENT;
    pd_params_default(s, r);
    std::ifstream in(path);
    if (!in.is_open()) return PD_ERR_FILE;
    std::string line, name, value;
    while (std::getline(in, line)) {
        line.erase(line.find_last_not_of(" \n\r\t") + 1);
        if (line.empty()) continue;
        if (line.find("//") != std::string::npos) continue;
        std::istringstream iss(line);
        name.clear();
        value.clear();
        iss >> name >> value;
        const char* v = value.c_str();
        if (name == "num_pd_particle") s->num_pd_particle = std::atoi(v);
        else if (name == "radius_pd_over_sph") s->pd_particle_radius = std::atof(v);
        else if (name == "boundary_min_x") s->boundary_min_x = std::atof(v);
        else if (name == "boundary_min_y") s->boundary_min_y = std::atof(v);
        else if (name == "boundary_min_z") s->boundary_min_z = std::atof(v);
        else if (name == "boundary_max_x") s->boundary_max_x = std::atof(v);
        else if (name == "boundary_max_y") s->boundary_max_y = std::atof(v);
        else if (name == "boundary_max_z") s->boundary_max_z = std::atof(v);
        else if (name == "sph_kernel_coeff") s->sph_kernel_coeff = std::atof(v);
        else if (name == "pd_kernel_coeff") s->pd_kernel_coeff = std::atof(v);
        else if (name == "sph_particle_mass") s->sph_particle_mass = std::atof(v);
        else if (name == "pd_particle_mass") s->pd_particle_mass = std::atof(v);
        else if (name == "adaptive_integration") r->adaptive_integration = std::atoi(v);
        else if (name == "gpu_device") r->gpu_device = std::atoi(v);
        else if (name == "steps_per_frame") r->step_per_frame = std::atoi(v);
        else if (name == "tube_radius") r->tube_radius = std::atoi(v);
        else if (name == "wall_thickness") r->wall_thickness = std::atoi(v);
        else if (name == "mesh_translation_x") r->mesh_translation_x = (float)std::atof(v);
        else if (name == "mesh_translation_y") r->mesh_translation_y = (float)std::atof(v);
        else if (name == "mesh_translation_z") r->mesh_translation_z = (float)std::atof(v);
        else if (name == "sph_initial_velocity") r->sph_initial_velocity = (float)std::atof(v);
        else if (name == "pd_stretch_limit_s0") r->pd_stretch_limit_s0 = (float)std::atof(v);
        else if (name == "pd_initial_velocity") r->pd_initial_velocity = (float)std::atof(v);
        else if (name == "steps_per_state") r->step_per_state = std::atoi(v);
        else if (name == "start_step") r->start_step = std::atoi(v);
        else if (name == "final_step") r->final_step = std::atoi(v);
        else if (name == "dump_density") r->dump_density = std::atoi(v);
        else if (name == "dump_velocity") r->dump_velocity = std::atoi(v);
        else if (name == "dump_activity") r->dump_activity = std::atoi(v);
        else if (name == "dump_pd_bond_list_top") r->dump_pd_bond_list_top = std::atoi(v);
        else if (name == "obj_file") {
            std::strncpy(r->obj_file, v, sizeof(r->obj_file) - 1);
        } else if (name == "saving_path") {
            std::strncpy(r->saving_path, v, sizeof(r->saving_path) - 1);
        } else if (name == "integrator") {
            r->integrator = (value == "implicit_euler") ? PD_IMPLICIT_EULER : PD_NEWMARK_BETA;
        }
        // num_sph_particle, sph_*_viscosity, sph_pd_slip: SPH only, ignored
    }
    return pd_params_derive(s, r);
}

extern "C" pd_status pd_solver_options_default(pd_solver_options* o)
{
    if (!o) return PD_ERR_INVALID_ARGUMENT;
    std::memset(o, 0, sizeof(*o));
    o->precision = PD_PRECISION_MIXED;
    o->contact_distance = 0.75 * 0.0005;
    o->contact_stiffness = 1.0e7;
    o->contact_volume = 0.0005 * 0.0005 * 0.0005;
    o->cg_relative_tolerance = 1e-20;
    o->cg_max_iterations = 100000;
    o->time_step_base = 1.0 / 8388608.0;
    o->time_step_min = 100;
    o->max_substep = 10;
    o->phase_in_steps = 30;
    o->pd_k = 5.0 * 2.94315e9;
    o->bond_stiffness = 0.0;
    o->gravity[0] = 0.0;
    o->gravity[1] = -9.8;
    o->gravity[2] = 0.0;
    o->restitution = 0.001;
    o->box_enabled = 1;
    o->stretch_a = 10.0;
    o->stretch_b = 9.0;
    o->alpha = 0.25;
    o->max_bonds_per_particle = 528;
    o->sphere_enabled = 0;
    o->lanes_per_particle = 0;
    o->cg_check_interval = 0;
    o->cg_loop = 0;
    o->preconditioner = 0;
    return PD_OK;
}

#include "glibc_rand.h"

using pdgb::GlibcRand;

extern "C" pd_status pd_sample_stretch_limits(float s0, int n, double* out)
{
    if (n < 0 || (n > 0 && !out)) return PD_ERR_INVALID_ARGUMENT;
    GlibcRand gen(1973);
    const double s0d = (double)s0;
    for (int p = 0; p < n; ++p) {
        // getstretch(): 12 frand() summed, minus 6, scaled (simulator.cu:802-822)
        double sum = 0.0;
        for (int k = 0; k < 12; ++k) sum += gen.next() / (double)2147483647;
        sum -= 6.0;
        out[p] = ((sum * 0.01 + 1.0) * s0d);
    }
    return PD_OK;
}

extern "C" pd_status pd_adaptive_decide(int has_broken, int ticks_base, int ticks_min, int max_substep, int* ticks,
                                        int* substep, int* rollback)
{
    if (!ticks || !substep || !rollback) return PD_ERR_INVALID_ARGUMENT;
    *rollback = 0;
    if (has_broken) {
        if (*ticks > ticks_min) {
            *ticks /= 2;
            *rollback = 1;
            return PD_OK;
        }
        *substep = 1;
    } else {
        if (*substep > 0) ++*substep;
        if (*substep >= max_substep) {
            *ticks *= 2;
            *substep = (*ticks >= ticks_base) ? 0 : 1;
        }
    }
    return PD_OK;
}
