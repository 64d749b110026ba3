// scene.cpp -- the reference's example Scene for the PD particles: an OBJ
// mesh scaled into the simulation box and filled with a lattice on the GPU
// (Scene::Scene, Scene::fillParticlesToMesh, Scene::initPeridynamicsParticles,
// src/examples/scene.cpp:18-135, 360-395, 537-598; OBJ reading of
// src/examples/cyTriMesh.h).
//
// The arithmetic of the placement follows the reference operation by
// operation, including its float/double mix (the mesh and its bounding box
// are float, cyPoint3f; the scale, shifts and lattice points double), so the
// same OBJ file and parameters give the same lattice and the same particles.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "glibc_rand.h"
#include "mesh.h"
#include "pd_gb300.h"

namespace pdgb {
void set_handleless_error(const std::string& msg);   // capi.cpp

namespace {

struct F3 {
    float x, y, z;
};

// cyTriMesh::LoadFromFileObj: "v x y z" vertices (float), "f" faces with
// 1-based indices (v, v/vt, v/vt/vn), polygons split into the fan
// (v0, v[k-1], v[k]); lines end at '\n' or '\r'.
bool load_obj(const char* path, std::vector<F3>& V, std::vector<int>& T, std::string& err)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        err = std::string("cannot open OBJ file ") + path;
        return false;
    }
    std::string text;
    char buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    std::fclose(f);
    size_t pos = 0;
    while (pos <= text.size()) {
        size_t end = text.find_first_of("\r\n", pos);
        if (end == std::string::npos) end = text.size();
        const std::string line = text.substr(pos, end - pos);
        pos = end + 1;
        if (line.size() >= 2 && line[0] == 'v' && (line[1] == ' ' || line[1] == '\t')) {
            F3 v{0.f, 0.f, 0.f};
            std::sscanf(line.c_str() + 2, "%f %f %f", &v.x, &v.y, &v.z);
            V.push_back(v);
        } else if (!line.empty() && line[0] == 'f') {
            int face[3] = {0, 0, 0};
            int facevert = -1;
            bool inspace = true;
            int type = 0;
            unsigned index = 0;
            std::vector<int> tris;
            for (size_t i = 2; i < line.size(); ++i) {
                const char c = line[i];
                if (c == ' ' || c == '\t') {
                    inspace = true;
                    continue;
                }
                if (inspace) {
                    inspace = false;
                    type = 0;
                    index = 0;
                    if (facevert < 2) {
                        ++facevert;
                    } else {   // next fan triangle: first vertex and the previous third
                        tris.insert(tris.end(), face, face + 3);
                        face[1] = face[2];
                    }
                }
                if (c == '/') {
                    ++type;
                    index = 0;
                }
                if (c >= '0' && c <= '9') {
                    index = index * 10 + (unsigned)(c - '0');
                    if (type == 0) face[facevert] = (int)(index - 1);
                }
            }
            if (facevert == 2) {
                tris.insert(tris.end(), face, face + 3);
                T.insert(T.end(), tris.begin(), tris.end());
            }
        }
        if (end == text.size()) break;
    }
    for (int t : T)
        if (t < 0 || t >= (int)V.size()) {
            err = "OBJ face index out of range";
            return false;
        }
    return true;
}

}  // namespace

class MeshScene {
public:
    std::vector<double> pos;   // double4 per particle, lattice order, before initPeridynamicsParticles
    int count = 0;
    pd_run_params run;
    double scale_factor = 1.0;
};

}  // namespace pdgb

struct pd_scene {
    pdgb::MeshScene* s;
};

namespace {
thread_local std::string g_scene_error;

pd_status scene_fail(const std::string& msg, pd_status st)
{
    g_scene_error = msg;
    pdgb::set_handleless_error(msg);
    return st;
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { cudaFree(p); }
};
}  // namespace

extern "C" {

pd_status pd_scene_create(pd_sim_params* sim, const pd_run_params* run, int jittered, unsigned jitter_seed,
                          pd_scene** out)
{
    using namespace pdgb;
    if (!sim || !run || !out) return PD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::vector<F3> V;
    std::vector<int> T;
    std::string err;
    if (!load_obj(run->obj_file, V, T, err)) return scene_fail(err, PD_ERR_FILE);
    if (V.empty() || T.empty()) return scene_fail("OBJ file has no triangles", PD_ERR_INVALID_ARGUMENT);
    if (!(sim->pd_particle_radius > 0)) return scene_fail("pd_particle_radius must be positive", PD_ERR_INVALID_ARGUMENT);
    // cyTriMesh::ComputeBoundingBox (float)
    F3 bmin = V[0], bmax = V[0];
    for (const F3& v : V) {
        if (bmin.x > v.x) bmin.x = v.x;
        if (bmin.y > v.y) bmin.y = v.y;
        if (bmin.z > v.z) bmin.z = v.z;
        if (bmax.x < v.x) bmax.x = v.x;
        if (bmax.y < v.y) bmax.y = v.y;
        if (bmax.z < v.z) bmax.z = v.z;
    }
    // Scene::Scene (scene.cpp:33-71): fit the mesh into half of 0.9 x the
    // smallest box extent, move its minimum corner to boundary_min
    const F3 diff{bmax.x - bmin.x, bmax.y - bmin.y, bmax.z - bmin.z};
    const double maxDiff = fmaxf(fmaxf(std::fabs(diff.x), std::fabs(diff.y)), std::fabs(diff.z));
    double scale = fminf(fminf((float)(sim->boundary_max_x - sim->boundary_min_x),
                               (float)(sim->boundary_max_y - sim->boundary_min_y)),
                         (float)(sim->boundary_max_z - sim->boundary_min_z)) * 0.9 / maxDiff;
    scale *= 0.5f;
    bmin.x = (float)(bmin.x * scale); bmin.y = (float)(bmin.y * scale); bmin.z = (float)(bmin.z * scale);
    bmax.x = (float)(bmax.x * scale); bmax.y = (float)(bmax.y * scale); bmax.z = (float)(bmax.z * scale);
    const double shift_x = sim->boundary_min_x - bmin.x;
    const double shift_y = sim->boundary_min_y - bmin.y;
    const double shift_z = sim->boundary_min_z - bmin.z;
    bmin.x = (float)(bmin.x + shift_x); bmax.x = (float)(bmax.x + shift_x);
    bmin.y = (float)(bmin.y + shift_y); bmax.y = (float)(bmax.y + shift_y);
    bmin.z = (float)(bmin.z + shift_z); bmax.z = (float)(bmax.z + shift_z);
    // Scene::createPeridynamicsGrid (scene.cpp:635-646)
    const double r = sim->pd_particle_radius;
    const int nx = (int)std::ceil((bmax.x - bmin.x) / (2.0f * r)) + 1;
    const int ny = (int)std::ceil((bmax.y - bmin.y) / (2.0f * r)) + 1;
    const int nz = (int)std::ceil((bmax.z - bmin.z) / (2.0f * r)) + 1;
    const long long total = (long long)nx * ny * nz;
    if (nx <= 0 || ny <= 0 || nz <= 0 || total >= (1ll << 31))
        return scene_fail("lattice too large for the mesh box and radius", PD_ERR_INVALID_ARGUMENT);
    // transformed vertices (double), triangles, and the triangles' bounding box
    std::vector<double> X(3 * V.size());
    for (size_t i = 0; i < V.size(); ++i) {
        X[3 * i] = (double)V[i].x * scale + shift_x;
        X[3 * i + 1] = (double)V[i].y * scale + shift_y;
        X[3 * i + 2] = (double)V[i].z * scale + shift_z;
    }
    const int ntri = (int)(T.size() / 3);
    MeshGrid M{};
    for (int k = 0; k < 3; ++k) {
        M.box_lo[k] = 1e300;
        M.box_hi[k] = -1e300;
    }
    for (int t : T)
        for (int k = 0; k < 3; ++k) {
            M.box_lo[k] = std::fmin(M.box_lo[k], X[3 * (size_t)t + k]);
            M.box_hi[k] = std::fmax(M.box_hi[k], X[3 * (size_t)t + k]);
        }
    // xy bins of the triangles (a +z ray from p can only cross triangles
    // whose xy bounding box contains p); ~4 triangles per bin on average
    const int nb_target = std::max(1, ntri / 4);
    const double wx = M.box_hi[0] - M.box_lo[0], wy = M.box_hi[1] - M.box_lo[1];
    int bx = std::max(1, (int)std::lround(std::sqrt((double)nb_target * (wx + 1e-300) / (wy + 1e-300))));
    bx = std::min(bx, 4096);
    int by = std::max(1, std::min(4096, (nb_target + bx - 1) / bx));
    M.bins_x = bx;
    M.bins_y = by;
    M.bin_x0 = M.box_lo[0];
    M.bin_y0 = M.box_lo[1];
    M.bin_inv_w = wx > 0 ? bx / wx : 0.0;
    M.bin_inv_h = wy > 0 ? by / wy : 0.0;
    auto bin_of = [](double v, double v0, double inv, int nb) {
        int b = (int)std::floor((v - v0) * inv);
        return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
    };
    std::vector<int> start((size_t)bx * by + 1, 0), list;
    std::vector<int> tb(4 * (size_t)ntri);
    for (int t = 0; t < ntri; ++t) {
        double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300};
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 2; ++k) {
                lo[k] = std::fmin(lo[k], X[3 * (size_t)T[3 * t + j] + k]);
                hi[k] = std::fmax(hi[k], X[3 * (size_t)T[3 * t + j] + k]);
            }
        tb[4 * t] = bin_of(lo[0], M.bin_x0, M.bin_inv_w, bx);
        tb[4 * t + 1] = bin_of(hi[0], M.bin_x0, M.bin_inv_w, bx);
        tb[4 * t + 2] = bin_of(lo[1], M.bin_y0, M.bin_inv_h, by);
        tb[4 * t + 3] = bin_of(hi[1], M.bin_y0, M.bin_inv_h, by);
        for (int y = tb[4 * t + 2]; y <= tb[4 * t + 3]; ++y)
            for (int x = tb[4 * t]; x <= tb[4 * t + 1]; ++x) ++start[(size_t)y * bx + x + 1];
    }
    for (size_t b = 0; b < (size_t)bx * by; ++b) start[b + 1] += start[b];
    list.assign((size_t)start[(size_t)bx * by], 0);
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int t = 0; t < ntri; ++t)
            for (int y = tb[4 * t + 2]; y <= tb[4 * t + 3]; ++y)
                for (int x = tb[4 * t]; x <= tb[4 * t + 1]; ++x) list[(size_t)fill[(size_t)y * bx + x]++] = t;
    }
    // lattice (Scene::fillParticlesToMesh, scene.cpp:537-598)
    const double spacing = 2 * r;
    M.lat_min[0] = bmin.x;
    M.lat_min[1] = bmin.y;
    M.lat_min[2] = bmin.z;
    M.spacing = spacing;
    M.nx = nx;
    M.ny = ny;
    M.nz = nz;
    M.clamp_lo[0] = bmin.x; M.clamp_lo[1] = bmin.y; M.clamp_lo[2] = bmin.z;
    M.clamp_hi[0] = bmax.x; M.clamp_hi[1] = bmax.y; M.clamp_hi[2] = bmax.z;
    std::vector<double> jit;
    if (jittered) {
        // (frand() * 2 - 1) * JITTER * radius, three per lattice point in loop order
        const double jitter = 0.01 * r;
        GlibcRand gen((int32_t)jitter_seed);
        jit.resize(3 * (size_t)total);
        for (size_t i = 0; i < jit.size(); ++i) {
            const double fr = gen.next() / (double)2147483647;
            jit[i] = (fr * 2.0f - 1.0f) * jitter;
        }
    }
    if (cudaSetDevice(run->gpu_device) != cudaSuccess) {
        cudaGetLastError();
        return scene_fail("no usable CUDA device", PD_ERR_NO_DEVICE);
    }
    DevBuf dv, dt, ds, dl, dj;
    cudaError_t e = cudaMalloc(&dv.p, sizeof(double) * X.size());
    if (e == cudaSuccess) e = cudaMalloc(&dt.p, sizeof(int) * T.size());
    if (e == cudaSuccess) e = cudaMalloc(&ds.p, sizeof(int) * start.size());
    if (e == cudaSuccess) e = cudaMalloc(&dl.p, sizeof(int) * std::max<size_t>(list.size(), 1));
    if (e == cudaSuccess && jittered) e = cudaMalloc(&dj.p, sizeof(double) * jit.size());
    if (e == cudaSuccess) e = cudaMemcpy(dv.p, X.data(), sizeof(double) * X.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt.p, T.data(), sizeof(int) * T.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ds.p, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !list.empty())
        e = cudaMemcpy(dl.p, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && jittered) e = cudaMemcpy(dj.p, jit.data(), sizeof(double) * jit.size(), cudaMemcpyHostToDevice);
    M.vtx = (const double*)dv.p;
    M.tri = (const int*)dt.p;
    M.bin_start = (const int*)ds.p;
    M.bin_tri = (const int*)dl.p;
    M.jitter = jittered ? (const double*)dj.p : nullptr;
    double* d_out = nullptr;
    long long count = 0;
    if (e == cudaSuccess) e = mesh_fill(M, &d_out, &count, 0);
    DevBuf dout;
    dout.p = d_out;
    std::unique_ptr<MeshScene> sc(new (std::nothrow) MeshScene());
    if (!sc) return PD_ERR_OUT_OF_MEMORY;
    if (e == cudaSuccess) {
        sc->pos.resize(4 * (size_t)count);
        if (count) e = cudaMemcpy(sc->pos.data(), d_out, sizeof(double) * 4 * (size_t)count, cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) {
        const std::string msg = std::string("scene fill: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return scene_fail(msg, e == cudaErrorMemoryAllocation ? PD_ERR_OUT_OF_MEMORY : PD_ERR_CUDA);
    }
    sc->count = (int)count;
    sc->run = *run;
    sc->scale_factor = sim->scaleFactor;
    sim->num_pd_particle = (int)count;
    pd_scene* h = new (std::nothrow) pd_scene{sc.release()};
    if (!h) return PD_ERR_OUT_OF_MEMORY;
    *out = h;
    return PD_OK;
}

pd_status pd_scene_particle_count(pd_scene* s, int* count)
{
    if (!s || !s->s || !count) return PD_ERR_INVALID_ARGUMENT;
    *count = s->s->count;
    return PD_OK;
}

pd_status pd_scene_init_pd_particles(pd_scene* s, int32_t* activity, double* pos4, double* vel4)
{
    if (!s || !s->s) return PD_ERR_INVALID_ARGUMENT;
    const pdgb::MeshScene& sc = *s->s;
    const int n = sc.count;
    if (n > 0 && (!activity || !pos4 || !vel4)) return PD_ERR_INVALID_ARGUMENT;
    // translation by mesh_translation / scaleFactor, no rotation (scene.cpp:371-386, 653-690)
    const double t[3] = {sc.run.mesh_translation_x / sc.scale_factor, sc.run.mesh_translation_y / sc.scale_factor,
                         sc.run.mesh_translation_z / sc.scale_factor};
    const double v0 = sc.run.pd_initial_velocity;
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) pos4[4 * (size_t)i + k] = sc.pos[4 * (size_t)i + k] + t[k];
        pos4[4 * (size_t)i + 3] = 0.0;
        for (int k = 0; k < 4; ++k) vel4[4 * (size_t)i + k] = v0;
        activity[i] = PD_ACTIVE;
    }
    return PD_OK;
}

pd_status pd_scene_destroy(pd_scene* s)
{
    if (!s) return PD_ERR_INVALID_ARGUMENT;
    delete s->s;
    delete s;
    return PD_OK;
}

const char* pd_scene_last_error_message(void) { return g_scene_error.c_str(); }

}  // extern "C"
