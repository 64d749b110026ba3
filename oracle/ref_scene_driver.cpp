// ref_scene_driver.cpp -- host driver of the reference's example Scene
// (src/examples/scene.cpp, with the mesh_query0.1 inside test and cyTriMesh
// OBJ reader), compiled from the reference tree by oracle/build_ref.sh into
// oracle/_ref/libpdscene.so.  TEST INFRASTRUCTURE ONLY: the source of the
// mesh-fill golden fixtures (tests/golden/make_mesh_golden.py).
#include <cstring>
#include <string>
#include <vector>

#include "core/monitor.h"
#include "scene.h"

// Monitor's logging statics used by Scene (the rest of Monitor is not needed)
const std::string Monitor::PADDING = "    ";
void Monitor::recordEvent(const char*) {}

// Scene(sim, run, arrangement) + initPeridynamicsParticles for an OBJ file and
// a simulation box; returns the particle count, fills out (4 doubles per
// particle, at most cap) when out is not null.  arrangement 0 REGULAR_GRID.
extern "C" int ref_scene_fill(const char* obj, const double* bmin, const double* bmax, double radius,
                              double scale_factor, const float* translation, float initial_velocity,
                              int arrangement, double* out, double* vel_out, int cap)
{
    SimulationParameters sp;
    std::memset(&sp, 0, sizeof(sp));
    RunningParameters rp;
    std::memset(&rp, 0, sizeof(rp));
    sp.num_pd_particle = 1;
    sp.boundary_min_x = bmin[0];
    sp.boundary_min_y = bmin[1];
    sp.boundary_min_z = bmin[2];
    sp.boundary_max_x = bmax[0];
    sp.boundary_max_y = bmax[1];
    sp.boundary_max_z = bmax[2];
    sp.pd_particle_radius = radius;
    sp.scaleFactor = scale_factor;
    rp.mesh_translation_x = translation[0];
    rp.mesh_translation_y = translation[1];
    rp.mesh_translation_z = translation[2];
    rp.pd_initial_velocity = initial_velocity;
    std::strncpy(rp.obj_file, obj, sizeof(rp.obj_file) - 1);
    Scene sc(sp, rp, arrangement ? Scene::JITTERED_GRID : Scene::REGULAR_GRID);
    const int n = sp.num_pd_particle;
    if (!out) return n;
    std::vector<int> act((size_t)n);
    std::vector<double4> pos((size_t)n), vel((size_t)n);
    sc.initPeridynamicsParticles(act.data(), pos.data(), vel.data());
    for (int i = 0; i < n && i < cap; ++i) {
        out[4 * i] = pos[i].x;
        out[4 * i + 1] = pos[i].y;
        out[4 * i + 2] = pos[i].z;
        out[4 * i + 3] = pos[i].w;
        if (vel_out) {
            vel_out[4 * i] = vel[i].x;
            vel_out[4 * i + 1] = vel[i].y;
            vel_out[4 * i + 2] = vel[i].z;
            vel_out[4 * i + 3] = vel[i].w;
        }
    }
    return n;
}
