// dataio.cpp -- DataIO of the reference (src/core/dataIO.cu): frames, the
// simulation-info files and checkpoints under RunningParameters::saving_path.
//
// Frames and info files are byte-compatible with the reference's readers:
//   <saving_path>/DATA/<VAR>/frame.<savedFrame>   raw host array of the
//       variable in caller order (DataIO::getDataAndWrite, dataIO.cu:98-124);
//       PD_POSITION is double4 scaled by scaleFactor (memory_manager.cu:274-298),
//       PD_VELOCITY double4, PD_ACTIVITY / PD_BOND_LIST_TOP /
//       PD_ORIGINAL_BOND_COUNT int32 (bond list tops are counts - 1);
//   <saving_path>/DATA/sim_info.dat   the reference's SimulationParameters
//       struct, raw (dataIO.cu:254-264; field order of parameters.h:16-88);
//   <saving_path>/DATA/viz_info.dat   its text summary (dataIO.cu:266-298).
// Which variables are written follows DataIO's saving map (dataIO.cu:30-63):
// positions always, velocities / activity / bond-list tops when dump_velocity /
// dump_activity / dump_pd_bond_list_top are set; the SPH folders are created
// as the reference does, and stay empty (no SPH particles).
//
// Checkpoints: the reference writes <saving_path>/STATE/state.<step> while it
// creates <saving_path>/DATA/STATE (dataIO.cu:162-164 vs 227-235), so its
// saveState fails unless STATE/ exists by chance; here the file goes to the
// folder that is created, DATA/STATE/state.<step>.  After the reference's
// leading savedFrame (size_t) the file holds this library's own layout: the
// device state in slot order, the step-loop state and the bond lists -- what
// a handle needs to continue a run bit for bit -- not the reference's full
// MemoryManager dump (whose 528 x 72-byte-per-particle system matrix this
// implementation never forms).
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "engine.h"

namespace pdgb {

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

namespace {

// Field order and types of the reference's SimulationParameters
// (parameters.h:16-88, real_t = double, definitions.h:18-39).
struct RefSimulationParameters {
    int num_total_particle, num_sph_particle, num_pd_particle;
    int num_cell_x, num_cell_y, num_cell_z, num_cells, num_clists;
    double cell_size;
    double sph_kernel_coeff, pd_kernel_coeff, sph_particle_mass, pd_particle_mass;
    double sph_sph_viscosity, sph_boundary_viscosity, sph_pd_slip;
    double boundary_min_x, boundary_min_y, boundary_min_z, boundary_max_x, boundary_max_y, boundary_max_z;
    double pd_min_x, pd_min_y, pd_min_z, pd_max_x, pd_max_y, pd_max_z;
    int boundaryPlaneSize, boundaryPlaneBottomIndex, boundaryPlaneBottomSize, boundaryPlaneTopIndex,
        boundaryPlaneTopSize, boundaryPlaneFrontIndex, boundaryPlaneFrontSize, boundaryPlaneBackIndex,
        boundaryPlaneBackSize, boundaryPlaneLeftSideIndex, boundaryPlaneLeftSideSize,
        boundaryPlaneRightSideIndex, boundaryPlaneRightSideSize;
    int pd_max_num_bonds, pd_time_step;
    double sph_kernel_smooth_length, sph_kernel_smooth_length_squared, sph_particle_radius, sph_kernel_poly6,
        sph_kernel_spiky, sph_rest_density;
    double pd_particle_radius, pd_horizon, pd_C_times_V, sph_pd_min_distance;
    double clockScale, scaleFactor;
};

constexpr char kStateMagic[16] = "PDGB300-STATE01";
constexpr unsigned kStateVersion = 1;

bool make_dir(const std::string& path)
{
    struct stat info;
    if (stat(path.c_str(), &info) == 0) return (info.st_mode & S_IFDIR) != 0;
    return mkdir(path.c_str(), 0775) == 0 || errno == EEXIST;
}

bool write_file(const std::string& path, const void* data, size_t bytes)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const size_t w = bytes ? std::fwrite(data, 1, bytes, f) : 0;
    return std::fclose(f) == 0 && w == bytes;
}

struct Writer {
    FILE* f;
    bool ok = true;
    template <typename T>
    void put(const T& v) { ok = ok && std::fwrite(&v, sizeof(T), 1, f) == 1; }
    void bytes(const void* p, size_t n) { ok = ok && (n == 0 || std::fwrite(p, 1, n, f) == n); }
};

struct Reader {
    FILE* f;
    bool ok = true;
    template <typename T>
    void get(T& v) { ok = ok && std::fread(&v, sizeof(T), 1, f) == 1; }
    void bytes(void* p, size_t n) { ok = ok && (n == 0 || std::fread(p, 1, n, f) == n); }
};

}  // namespace

// DataIO::writeSimulationParameter (dataIO.cu:251-299)
pd_status Engine::dataio_write_sim_info()
{
    const std::string root = run_.saving_path;
    if (!make_dir(root) || !make_dir(root + "/DATA")) {
        err_ = "DataIO: cannot create " + root + "/DATA";
        return PD_ERR_FILE;
    }
    RefSimulationParameters r;
    std::memset(&r, 0, sizeof(r));
    r.num_total_particle = n_;
    r.num_sph_particle = 0;
    r.num_pd_particle = n_;
    r.num_cell_x = sim_.num_cell_x;
    r.num_cell_y = sim_.num_cell_y;
    r.num_cell_z = sim_.num_cell_z;
    r.num_cells = sim_.num_cells;
    r.cell_size = sim_.cell_size;
    r.sph_kernel_coeff = sim_.sph_kernel_coeff;
    r.pd_kernel_coeff = sim_.pd_kernel_coeff;
    r.sph_particle_mass = sim_.sph_particle_mass;
    r.pd_particle_mass = sim_.pd_particle_mass;
    r.boundary_min_x = sim_.boundary_min_x;
    r.boundary_min_y = sim_.boundary_min_y;
    r.boundary_min_z = sim_.boundary_min_z;
    r.boundary_max_x = sim_.boundary_max_x;
    r.boundary_max_y = sim_.boundary_max_y;
    r.boundary_max_z = sim_.boundary_max_z;
    if (n_ > 0) {   // pd_min/max: the bounding box of the initial positions (Scene)
        r.pd_min_x = r.pd_min_y = r.pd_min_z = 1e300;
        r.pd_max_x = r.pd_max_y = r.pd_max_z = -1e300;
        for (int i = 0; i < n_; ++i) {
            const double* p = &h_pos_[4 * (size_t)i];
            r.pd_min_x = std::min(r.pd_min_x, p[0]); r.pd_max_x = std::max(r.pd_max_x, p[0]);
            r.pd_min_y = std::min(r.pd_min_y, p[1]); r.pd_max_y = std::max(r.pd_max_y, p[1]);
            r.pd_min_z = std::min(r.pd_min_z, p[2]); r.pd_max_z = std::max(r.pd_max_z, p[2]);
        }
    }
    r.pd_max_num_bonds = sim_.pd_max_num_bonds;
    r.pd_time_step = ticks_;
    r.sph_particle_radius = sim_.sph_particle_radius;
    r.pd_particle_radius = sim_.pd_particle_radius;
    r.pd_horizon = sim_.pd_horizon;
    r.pd_C_times_V = sim_.pd_C_times_V;
    r.clockScale = clock_scale_;
    r.scaleFactor = sim_.scaleFactor;
    if (!write_file(root + "/DATA/sim_info.dat", &r, sizeof(r))) {
        err_ = "DataIO: cannot write sim_info.dat";
        return PD_ERR_FILE;
    }
    std::ofstream viz(root + "/DATA/viz_info.dat", std::ofstream::out);
    if (!viz.is_open()) {
        err_ = "DataIO: cannot write viz_info.dat";
        return PD_ERR_FILE;
    }
    viz << "num_total_particle " << r.num_total_particle << std::endl;
    viz << "num_sph_particle " << r.num_sph_particle << std::endl;
    viz << "num_pd_particle " << r.num_pd_particle << std::endl;
    viz << "sph_kernel_coeff " << r.sph_kernel_coeff << std::endl;
    viz << "pd_kernel_coeff " << r.pd_kernel_coeff << std::endl;
    viz << "sph_particle_mass " << r.sph_particle_mass << std::endl;
    viz << "pd_particle_mass " << r.pd_particle_mass << std::endl;
    viz << "sph_sph_viscosity " << r.sph_sph_viscosity << std::endl;
    viz << "sph_boundary_viscosity " << r.sph_boundary_viscosity << std::endl;
    viz << "sph_pd_slip " << r.sph_pd_slip << std::endl;
    viz << "boundary_min_x " << r.boundary_min_x << std::endl;
    viz << "boundary_min_y " << r.boundary_min_y << std::endl;
    viz << "boundary_min_z " << r.boundary_min_z << std::endl;
    viz << "boundary_max_x " << r.boundary_max_x << std::endl;
    viz << "boundary_max_y " << r.boundary_max_y << std::endl;
    viz << "boundary_max_z " << r.boundary_max_z << std::endl;
    viz << "sph_particle_radius " << r.sph_particle_radius << std::endl;
    viz << "sph_rest_density " << r.sph_rest_density << std::endl;
    viz << "pd_particle_radius " << r.pd_particle_radius << std::endl;
    viz << "pd_horizon " << r.pd_horizon << std::endl;
    viz << "scaleFactor " << r.scaleFactor << std::endl;
    wrote_sim_info_ = true;
    return PD_OK;
}

// DataIO::getDataAndWrite (dataIO.cu:82-124) with the folders of
// createOutputFolders (dataIO.cu:207-249)
pd_status Engine::dataio_write_frame()
{
    if (!ready_) {
        err_ = "DataIO: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    const std::string data = std::string(run_.saving_path) + "/DATA";
    if (!wrote_sim_info_) {
        pd_status s = dataio_write_sim_info();
        if (s != PD_OK) return s;
    }
    std::vector<std::string> dirs = {"SPH_POSITION", "PD_POSITION"};
    if (run_.dump_velocity) dirs.insert(dirs.end(), {"SPH_VELOCITY", "PD_VELOCITY"});
    if (run_.dump_activity) dirs.insert(dirs.end(), {"SPH_ACTIVITY", "PD_ACTIVITY"});
    if (run_.dump_density) dirs.insert(dirs.end(), {"SPH_SORTED_POSITION", "SPH_SORTED_NORMALIZED_DENSITY"});
    if (run_.dump_pd_bond_list_top) dirs.insert(dirs.end(), {"PD_ORIGINAL_BOND_COUNT", "PD_BOND_LIST_TOP"});
    bool ok = make_dir(data + "/STATE");
    for (const auto& d : dirs) ok = ok && make_dir(data + "/" + d);
    if (!ok) {
        err_ = "DataIO: cannot create the output folders under " + data;
        return PD_ERR_FILE;
    }
    const std::string suffix = "/frame." + std::to_string(saved_frame_);
    const size_t N = (size_t)n_;
    auto write_int_var = [&](const char* name, const std::vector<int32_t>& v) -> pd_status {
        if (!write_file(data + "/" + name + suffix, v.data(), sizeof(int32_t) * v.size())) {
            err_ = std::string("DataIO: cannot write ") + name + suffix;
            return PD_ERR_FILE;
        }
        return PD_OK;
    };
    // variables in the reference's enum order (memory_manager.h:30-60)
    if (run_.dump_activity && N) {
        std::vector<int32_t> a(N);
        pd_status s = get(PD_VAR_ACTIVITY, a.data(), sizeof(int32_t) * N);
        if (s == PD_OK) s = write_int_var("PD_ACTIVITY", a);
        if (s != PD_OK) return s;
    }
    if (N) {
        std::vector<double> x(4 * N);
        pd_status s = get(PD_VAR_POSITION_SCALED, x.data(), sizeof(double) * 4 * N);
        if (s != PD_OK) return s;
        if (!write_file(data + "/PD_POSITION" + suffix, x.data(), sizeof(double) * 4 * N)) {
            err_ = "DataIO: cannot write PD_POSITION" + suffix;
            return PD_ERR_FILE;
        }
        if (run_.dump_velocity) {
            s = get(PD_VAR_VELOCITY, x.data(), sizeof(double) * 4 * N);
            if (s != PD_OK) return s;
            if (!write_file(data + "/PD_VELOCITY" + suffix, x.data(), sizeof(double) * 4 * N)) {
                err_ = "DataIO: cannot write PD_VELOCITY" + suffix;
                return PD_ERR_FILE;
            }
        }
    }
    if (run_.dump_pd_bond_list_top && N) {
        std::vector<int32_t> top(N);
        for (size_t i = 0; i < N; ++i) top[i] = cnt_init_[(size_t)inv_[i]] - 1;
        pd_status s = write_int_var("PD_ORIGINAL_BOND_COUNT", top);
        if (s != PD_OK) return s;
        s = get(PD_VAR_BOND_COUNT, top.data(), sizeof(int32_t) * N);
        if (s != PD_OK) return s;
        for (auto& t : top) t -= 1;
        s = write_int_var("PD_BOND_LIST_TOP", top);
        if (s != PD_OK) return s;
    }
    return PD_OK;
}

// DataIO::saveState (dataIO.cu:150-175), written to DATA/STATE
pd_status Engine::dataio_save_state(size_t timestep)
{
    if (!ready_) {
        err_ = "DataIO: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    pd_status s = dataio_write_sim_info();
    if (s != PD_OK) return s;
    const std::string dir = std::string(run_.saving_path) + "/DATA/STATE";
    if (!make_dir(dir)) {
        err_ = "DataIO: cannot create " + dir;
        return PD_ERR_FILE;
    }
    CK(cudaSetDevice(device_), "cudaSetDevice");
    CK(cudaStreamSynchronize(stream_), "state sync");
    const size_t N = (size_t)n_, slots = (size_t)std::max<long long>(total_slots_, 0);
    const size_t real = fp64_ ? sizeof(double) : sizeof(float);
    auto fetch = [&](const void* dev, size_t bytes, std::vector<char>& out) -> cudaError_t {
        out.resize(bytes);
        if (!bytes) return cudaSuccess;
        return cudaMemcpy(out.data(), dev, bytes, cudaMemcpyDeviceToHost);
    };
    const std::string path = dir + "/state." + std::to_string(timestep);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err_ = "DataIO: cannot write " + path;
        return PD_ERR_FILE;
    }
    Writer w{f};
    w.put(saved_frame_);
    w.bytes(kStateMagic, sizeof(kStateMagic));
    w.put(kStateVersion);
    w.put((int32_t)n_);
    w.put((int64_t)total_slots_);
    w.put((int32_t)(fp64_ ? 1 : 0));
    w.put((int32_t)step_);
    w.put((int32_t)substep_);
    w.put((int32_t)ticks_);
    w.put(clock_scale_);
    w.put(sim_time_);
    w.put((int32_t)(cg_converged_ ? 1 : 0));
    w.put((int64_t)total_iters_);
    w.put((int32_t)last_iters_);
    w.put(last_res_);
    w.put(last_tol_);
    w.bytes(perm_.data(), sizeof(int32_t) * N);
    w.bytes(cnt_init_.data(), sizeof(int32_t) * N);
    struct Arr {
        const void* dev;
        size_t bytes;
    };
    std::vector<Arr> arrs = {
        {S_.x64, sizeof(dbl4) * N},      {S_.v64, sizeof(dbl4) * N},       {S_.X64, sizeof(dbl4) * N},
        {S_.x64_bk, sizeof(dbl4) * N},   {S_.v64_bk, sizeof(dbl4) * N},    {S_.st, sizeof(double) * N},
        {S_.ost, sizeof(double) * N},    {S_.nst, sizeof(double) * N},     {S_.act, sizeof(uint8_t) * N},
        {S_.row_ptr, sizeof(int) * (N + 1)}, {S_.cnt, sizeof(int) * N},    {S_.cnt_bk, sizeof(int) * N},
        {S_.col, sizeof(int) * slots},   {S_.sol, 4 * real * N},
    };
    if (!fp64_) {
        arrs.push_back({S_.inv_d0, sizeof(float) * slots});
        arrs.push_back({S_.d0sq, sizeof(float2) * slots});
    }
    std::vector<char> buf;
    for (const Arr& a : arrs) {
        const cudaError_t e = fetch(a.dev, a.bytes, buf);
        if (e != cudaSuccess) {
            std::fclose(f);
            return cuda_fail(e, "DataIO: download state");
        }
        w.bytes(buf.data(), a.bytes);
    }
    const bool closed = std::fclose(f) == 0;
    if (!w.ok || !closed) {
        err_ = "DataIO: short write to " + path;
        return PD_ERR_FILE;
    }
    return PD_OK;
}

// DataIO::loadState (dataIO.cu:178-203): a handle made ready on the same
// scene (same particle count and bond structure) continues the saved run.
pd_status Engine::dataio_load_state(size_t timestep)
{
    if (!ready_) {
        err_ = "DataIO: make_ready has not run (load a state into a handle made ready on the same scene)";
        return PD_ERR_NOT_READY;
    }
    const std::string path = std::string(run_.saving_path) + "/DATA/STATE/state." + std::to_string(timestep);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err_ = "DataIO: cannot open " + path;
        return PD_ERR_FILE;
    }
    Reader r{f};
    size_t frame = 0;
    char magic[16];
    unsigned version = 0;
    int32_t n = 0, prec = 0, step = 0, substep = 0, ticks = 0, conv = 0, last_iters = 0;
    int64_t slots = 0, total_iters = 0;
    double cs = 0, t = 0, last_res = 0, last_tol = 0;
    r.get(frame);
    r.bytes(magic, sizeof(magic));
    r.get(version);
    r.get(n);
    r.get(slots);
    r.get(prec);
    r.get(step);
    r.get(substep);
    r.get(ticks);
    r.get(cs);
    r.get(t);
    r.get(conv);
    r.get(total_iters);
    r.get(last_iters);
    r.get(last_res);
    r.get(last_tol);
    if (!r.ok || std::memcmp(magic, kStateMagic, sizeof(kStateMagic)) != 0 || version != kStateVersion) {
        std::fclose(f);
        err_ = "DataIO: " + path + " is not a state file of this library";
        return PD_ERR_FILE;
    }
    if (n != n_ || slots != total_slots_ || prec != (fp64_ ? 1 : 0)) {
        std::fclose(f);
        err_ = "DataIO: inconsistent number of particles / bond slots / precision with the saved state";
        return PD_ERR_STATE;
    }
    const size_t N = (size_t)n_, nslots = (size_t)std::max<long long>(total_slots_, 0);
    const size_t real = fp64_ ? sizeof(double) : sizeof(float);
    std::vector<int32_t> perm(N), cinit(N);
    r.bytes(perm.data(), sizeof(int32_t) * N);
    r.bytes(cinit.data(), sizeof(int32_t) * N);
    struct Arr {
        void* dev;
        size_t bytes;
    };
    std::vector<Arr> arrs = {
        {S_.x64, sizeof(dbl4) * N},      {S_.v64, sizeof(dbl4) * N},       {S_.X64, sizeof(dbl4) * N},
        {S_.x64_bk, sizeof(dbl4) * N},   {S_.v64_bk, sizeof(dbl4) * N},    {S_.st, sizeof(double) * N},
        {S_.ost, sizeof(double) * N},    {S_.nst, sizeof(double) * N},     {S_.act, sizeof(uint8_t) * N},
        {S_.row_ptr, sizeof(int) * (N + 1)}, {S_.cnt, sizeof(int) * N},    {S_.cnt_bk, sizeof(int) * N},
        {S_.col, sizeof(int) * nslots},  {S_.sol, 4 * real * N},
    };
    if (!fp64_) {
        arrs.push_back({S_.inv_d0, sizeof(float) * nslots});
        arrs.push_back({S_.d0sq, sizeof(float2) * nslots});
    }
    CK(cudaSetDevice(device_), "cudaSetDevice");
    CK(cudaStreamSynchronize(stream_), "state sync");
    std::vector<char> buf;
    for (const Arr& a : arrs) {
        buf.resize(a.bytes);
        r.bytes(buf.data(), a.bytes);
        if (!r.ok) break;
        if (a.bytes) {
            const cudaError_t e = cudaMemcpy(a.dev, buf.data(), a.bytes, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                std::fclose(f);
                return cuda_fail(e, "DataIO: upload state");
            }
        }
    }
    std::fclose(f);
    if (!r.ok) {
        err_ = "DataIO: " + path + " is truncated";
        return PD_ERR_FILE;
    }
    CK(cudaMemcpy(d_perm_, perm.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice), "upload perm");
    // the lattice product's tables follow this handle's slot order: a state
    // saved in another order continues on the gather product
    const bool same_order = std::equal(perm.begin(), perm.end(), perm_.begin());
    perm_.assign(perm.begin(), perm.end());
    cnt_init_.assign(cinit.begin(), cinit.end());
    for (size_t i = 0; i < N; ++i) inv_[(size_t)perm_[i]] = (int)i;
    saved_frame_ = frame;
    step_ = step;
    substep_ = substep;
    ticks_ = ticks;
    clock_scale_ = cs;
    sim_time_ = t;
    cg_converged_ = conv != 0;
    total_iters_ = total_iters;
    last_iters_ = last_iters;
    last_res_ = last_res;
    last_tol_ = last_tol;
    predicted_iters_ = 0;
    hist_reset();   // the projection history belongs to the state that was replaced
    retries_ = 0;
    // derived device data: FP32 positions, tile local indices
    const StepParams P = step_params();
    if (!fp64_ && n_ > 0) {
        launch_refresh(fp64_, P, S_, L_, stream_);
        launch_stretch_limits(S_, (int)std::min<long long>(((long long)n_ + kBlock - 1) / kBlock, 4096), stream_);
        launches_ += 2;
        if (S_.lidx && S_.n_tiles > 0) {
            int max_halo = 0;
            CK(build_tiles(S_, n_, &max_halo, stream_), "rebuild tiles");
            S_.halo_cap = std::min(max_halo, kMaxHaloCap);
        }
    }
    if (lat_ok_ && !same_order) {
        lattice_free(&latb_);
        lat_ = LatticeParams{};
        lat_ok_ = false;
        lat_fixed_built_ = false;
        if (d_p2_) cudaFree(d_p2_);
        d_p2_ = nullptr;
        if (L_.lattice) {
            L_.lattice = 0;
            L_.lat = nullptr;
            L_.lanes = 8;
            L_.unroll = 1;
            L_.grid_bonds = grid_for_rows(8, row_kernel_blocks_per_sm(fp64_, 8, 1));
            lay_g_ = lay_u_ = 1;
        }
    }
    lattice_resync(true);
    last_params_ = P;
    CK(cudaStreamSynchronize(stream_), "state sync");
    return PD_OK;
}

}  // namespace pdgb

struct pd_handle {
    pdgb::Engine* eng;
};

extern "C" {

pd_status pd_dataio_get_data_and_write(pd_handle* h)
{
    if (!h || !h->eng) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->dataio_write_frame();
}

pd_status pd_dataio_new_frame(pd_handle* h)
{
    if (!h || !h->eng) return PD_ERR_INVALID_ARGUMENT;
    h->eng->dataio_new_frame();
    return PD_OK;
}

pd_status pd_dataio_saved_frame(pd_handle* h, size_t* frame)
{
    if (!h || !h->eng || !frame) return PD_ERR_INVALID_ARGUMENT;
    *frame = h->eng->dataio_saved_frame();
    return PD_OK;
}

pd_status pd_dataio_save_state(pd_handle* h, size_t timestep)
{
    if (!h || !h->eng) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->dataio_save_state(timestep);
}

pd_status pd_dataio_load_state(pd_handle* h, size_t timestep)
{
    if (!h || !h->eng) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->dataio_load_state(timestep);
}

}  // extern "C"
