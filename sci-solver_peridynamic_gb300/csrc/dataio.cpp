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

#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
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
        // no checkpoint of this library's layout: the reference's own
        // STATE/state.<step>, if there is one
        FILE* g = std::fopen(ref_state_path(timestep).c_str(), "rb");
        if (g) {
            std::fclose(g);
            return dataio_load_state_reference(timestep);
        }
        err_ = "DataIO: cannot open " + path + " (nor " + ref_state_path(timestep) + ")";
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

// ---- the reference's checkpoint layout -----------------------------------------------
// DataIO::saveState / loadState (dataIO.cu:123-198): savedFrame (size_t), then
// every MemoryManager array (memory_manager.h:29-90) in enum order, each with
// the size memory_manager.cu:16-178 gives it (real_t = double,
// definitions.h:33-39; MAX_PD_BOND_COUNT 528; Mat3x3 = 72 bytes; Clist = 136
// ints, definitions.h:99,137-147).  Positions (SPH and PD, sorted and original
// PD positions) are stored multiplied by scaleFactor (downloadFromDevice,
// memory_manager.cu:274-298).  The counts that size the arrays come from
// DATA/sim_info.dat of the same run (saveState writes it first, loadState
// reads it first).
namespace {

enum RefVar : int {
    R_SPH_TIMESTEP = 0, R_SPH_ACTIVITY, R_SPH_VALIDITY, R_SPH_POSITION, R_SPH_VELOCITY, R_SPH_FORCE,
    R_SPH_SORTED_POSITION, R_SPH_SORTED_VELOCITY, R_SPH_SORTED_DENSITY, R_SPH_SORTED_DENSITY_NORMALIZED,
    R_SPH_SORTED_PRESSURE, R_SPH_BOUNDARY_POSITION, R_PD_ACTIVITY, R_PD_POSITION, R_PD_POSITION_BACKUP,
    R_PD_VELOCITY, R_PD_VELOCITY_BACKUP, R_PD_FORCE, R_PD_SORTED_POSITION, R_PD_SORTED_VELOCITY,
    R_PD_ORIGINAL_POSITION, R_PD_ORIGINAL_STRETCH, R_PD_ORIGINAL_BOND_LIST_TOP, R_PD_STRETCH, R_PD_NEW_STRETCH,
    R_PD_BOND_LIST, R_PD_BOND_LIST_TOP, R_PD_BOND_LIST_TOP_BACKUP, R_PD_CLIST, R_PD_SYSTEM_MATRIX,
    R_PD_SYSTEM_VECTOR, R_PD_SYSTEM_SOLUTION, R_PD_HAS_BROKEN_BOND, R_CELL_PARTICLE_TYPE,
    R_SPH_PARTICLE_TO_CELL_HASH, R_SPH_PARTICLE_UNSORTED_INDEX, R_SPH_CELL_START_INDEX, R_SPH_CELL_END_INDEX,
    R_PD_PARTICLE_TO_CELL_HASH, R_PD_PARTICLE_UNSORTED_INDEX, R_PD_CELL_START_INDEX, R_PD_CELL_END_INDEX,
    R_NUM_VARIABLES
};
constexpr long long kRefMaxBonds = 528;
constexpr long long kRefMat3x3 = 72;
constexpr long long kRefClist = (128 + 1 + 7) * 4;

long long ref_var_bytes(int v, const RefSimulationParameters& r)
{
    const long long sph = r.num_sph_particle, pd = r.num_pd_particle, cells = r.num_cells;
    const long long P = r.boundaryPlaneSize;
    switch (v) {
    case R_SPH_TIMESTEP: case R_SPH_ACTIVITY: case R_SPH_VALIDITY:
    case R_SPH_PARTICLE_TO_CELL_HASH: case R_SPH_PARTICLE_UNSORTED_INDEX: return 4 * sph;
    case R_SPH_POSITION: case R_SPH_VELOCITY: case R_SPH_FORCE: case R_SPH_SORTED_POSITION:
    case R_SPH_SORTED_VELOCITY: return 32 * sph;
    case R_SPH_SORTED_DENSITY: case R_SPH_SORTED_DENSITY_NORMALIZED: case R_SPH_SORTED_PRESSURE: return 8 * sph;
    case R_SPH_BOUNDARY_POSITION: return 32 * (2 * (P + 2) * (P + 2) + 4 * P * (P + 1));
    case R_PD_ACTIVITY: case R_PD_ORIGINAL_BOND_LIST_TOP: case R_PD_BOND_LIST_TOP: case R_PD_BOND_LIST_TOP_BACKUP:
    case R_PD_PARTICLE_TO_CELL_HASH: case R_PD_PARTICLE_UNSORTED_INDEX: return 4 * pd;
    case R_PD_POSITION: case R_PD_POSITION_BACKUP: case R_PD_VELOCITY: case R_PD_VELOCITY_BACKUP: case R_PD_FORCE:
    case R_PD_SORTED_POSITION: case R_PD_SORTED_VELOCITY: case R_PD_ORIGINAL_POSITION: case R_PD_SYSTEM_VECTOR:
    case R_PD_SYSTEM_SOLUTION: return 32 * pd;
    case R_PD_ORIGINAL_STRETCH: case R_PD_STRETCH: case R_PD_NEW_STRETCH: return 8 * pd;
    case R_PD_BOND_LIST: return 4 * pd * kRefMaxBonds;
    case R_PD_CLIST: return kRefClist * (long long)r.num_clists;
    case R_PD_SYSTEM_MATRIX: return pd * kRefMaxBonds * kRefMat3x3;
    case R_PD_HAS_BROKEN_BOND: return 4;
    case R_CELL_PARTICLE_TYPE: case R_SPH_CELL_START_INDEX: case R_SPH_CELL_END_INDEX: case R_PD_CELL_START_INDEX:
    case R_PD_CELL_END_INDEX: return 4 * cells;
    default: return 0;
    }
}

long long ref_var_offset(int v, const RefSimulationParameters& r)
{
    long long off = (long long)sizeof(size_t);   // savedFrame
    for (int k = 0; k < v; ++k) off += ref_var_bytes(k, r);
    return off;
}

}  // namespace

std::string Engine::ref_state_path(size_t timestep) const
{
    return std::string(run_.saving_path) + "/STATE/state." + std::to_string(timestep);
}

// The reference's layout, written to STATE/state.<step> as its saveState
// writes it (that folder is created here; the reference assumes it exists).
// Arrays this engine does not hold (SPH, cell lists, contact lists) are
// zero-filled; the system matrix is left as a hole of the right length (the
// reference recomputes it every step; on file systems with sparse files it
// takes no space).  The bond list of each particle is its live bonds, then the
// bonds broken since the adaptive scheme's backup, then the earlier broken
// ones, in slot j * num_pd_particle + particle.
pd_status Engine::dataio_save_state_reference(size_t timestep)
{
    if (!ready_) {
        err_ = "DataIO: make_ready has not run";
        return PD_ERR_NOT_READY;
    }
    pd_status s = dataio_write_sim_info();
    if (s != PD_OK) return s;
    const std::string dir = std::string(run_.saving_path) + "/STATE";
    if (!make_dir(dir)) {
        err_ = "DataIO: cannot create " + dir;
        return PD_ERR_FILE;
    }
    RefSimulationParameters r;
    {
        FILE* fi = std::fopen((std::string(run_.saving_path) + "/DATA/sim_info.dat").c_str(), "rb");
        Reader rd{fi};
        if (fi) {
            rd.get(r);
            std::fclose(fi);
        }
        if (!fi || !rd.ok) {
            err_ = "DataIO: cannot read back DATA/sim_info.dat";
            return PD_ERR_FILE;
        }
    }
    CK(cudaSetDevice(device_), "cudaSetDevice");
    CK(cudaStreamSynchronize(stream_), "state sync");
    const size_t N = (size_t)n_;
    const double sf = sim_.scaleFactor;
    // caller-order arrays
    std::vector<double> pos(4 * N), pos_bk(4 * N), vel(4 * N), vel_bk(4 * N), opos(4 * N), force(4 * N), rhs(4 * N),
        sol(4 * N), st(N), ost(N), nst(N);
    s = get(PD_VAR_POSITION, pos.data(), pos.size() * sizeof(double));
    if (s == PD_OK) s = download_scatter((const double*)S_.x64_bk, pos_bk.data(), 4, N);
    if (s == PD_OK) s = get(PD_VAR_VELOCITY, vel.data(), vel.size() * sizeof(double));
    if (s == PD_OK) s = download_scatter((const double*)S_.v64_bk, vel_bk.data(), 4, N);
    if (s == PD_OK) s = get(PD_VAR_ORIGINAL_POSITION, opos.data(), opos.size() * sizeof(double));
    if (s == PD_OK) s = get(PD_VAR_FORCE, force.data(), force.size() * sizeof(double));
    if (s == PD_OK) s = export_vec4(S_.rhs, !fp64_, rhs.data());
    if (s == PD_OK) s = get(PD_VAR_SOLUTION, sol.data(), sol.size() * sizeof(double));
    if (s == PD_OK) s = get(PD_VAR_STRETCH, st.data(), st.size() * sizeof(double));
    if (s == PD_OK) s = get(PD_VAR_ORIGINAL_STRETCH, ost.data(), ost.size() * sizeof(double));
    if (s == PD_OK) s = get(PD_VAR_NEW_STRETCH, nst.data(), nst.size() * sizeof(double));
    if (s != PD_OK) return s;
    std::vector<int> rp(N + 1), cnt(N), cbk(N), col((size_t)std::max<long long>(total_slots_, 1));
    CK(cudaMemcpy(rp.data(), S_.row_ptr, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost), "download rp");
    if (N) {
        CK(cudaMemcpy(cnt.data(), S_.cnt, sizeof(int) * N, cudaMemcpyDeviceToHost), "download cnt");
        CK(cudaMemcpy(cbk.data(), S_.cnt_bk, sizeof(int) * N, cudaMemcpyDeviceToHost), "download cnt");
    }
    if (total_slots_ > 0)
        CK(cudaMemcpy(col.data(), S_.col, sizeof(int) * (size_t)total_slots_, cudaMemcpyDeviceToHost), "download col");
    for (size_t i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            pos[4 * i + k] *= sf;
            opos[4 * i + k] *= sf;
        }
    const std::string path = ref_state_path(timestep);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err_ = "DataIO: cannot write " + path;
        return PD_ERR_FILE;
    }
    Writer w{f};
    w.put(saved_frame_);
    std::vector<char> zeros;
    auto zero_fill = [&](long long bytes) {
        zeros.assign((size_t)std::min<long long>(bytes, 1 << 20), 0);
        for (long long left = bytes; left > 0 && w.ok; left -= (long long)zeros.size())
            w.bytes(zeros.data(), (size_t)std::min<long long>(left, (long long)zeros.size()));
    };
    std::vector<int32_t> ibuf;
    for (int v = 0; v < R_NUM_VARIABLES && w.ok; ++v) {
        const long long bytes = ref_var_bytes(v, r);
        const double* d4 = nullptr;
        switch (v) {
        case R_PD_POSITION: case R_PD_SORTED_POSITION: d4 = pos.data(); break;
        case R_PD_POSITION_BACKUP: d4 = pos_bk.data(); break;
        case R_PD_VELOCITY: case R_PD_SORTED_VELOCITY: d4 = vel.data(); break;
        case R_PD_VELOCITY_BACKUP: d4 = vel_bk.data(); break;
        case R_PD_FORCE: d4 = force.data(); break;
        case R_PD_ORIGINAL_POSITION: d4 = opos.data(); break;
        case R_PD_SYSTEM_VECTOR: d4 = rhs.data(); break;
        case R_PD_SYSTEM_SOLUTION: d4 = sol.data(); break;
        default: break;
        }
        if (d4) {
            w.bytes(d4, sizeof(double) * 4 * N);
            continue;
        }
        switch (v) {
        case R_PD_ACTIVITY: w.bytes(h_act_.data(), sizeof(int32_t) * N); break;
        case R_PD_ORIGINAL_STRETCH: w.bytes(ost.data(), sizeof(double) * N); break;
        case R_PD_STRETCH: w.bytes(st.data(), sizeof(double) * N); break;
        case R_PD_NEW_STRETCH: w.bytes(nst.data(), sizeof(double) * N); break;
        case R_PD_ORIGINAL_BOND_LIST_TOP: case R_PD_BOND_LIST_TOP: case R_PD_BOND_LIST_TOP_BACKUP:
            ibuf.assign(N, 0);
            for (size_t o = 0; o < N; ++o) {
                const int sl = inv_[o];
                ibuf[o] = (v == R_PD_ORIGINAL_BOND_LIST_TOP ? cnt_init_[sl] : v == R_PD_BOND_LIST_TOP ? cnt[sl] : cbk[sl]) - 1;
            }
            w.bytes(ibuf.data(), sizeof(int32_t) * N);
            break;
        case R_PD_BOND_LIST:
            ibuf.assign((size_t)kRefMaxBonds * N, 0);
            for (size_t o = 0; o < N; ++o) {
                const int sl = inv_[o];
                const int all = cnt_init_[sl];
                for (int j = 0; j < all && j < kRefMaxBonds; ++j) ibuf[(size_t)j * N + o] = perm_[col[rp[sl] + j]];
            }
            w.bytes(ibuf.data(), sizeof(int32_t) * ibuf.size());
            break;
        case R_PD_HAS_BROKEN_BOND: {
            const int32_t hb = 0;
            w.bytes(&hb, sizeof(hb));
            break;
        }
        case R_PD_SYSTEM_MATRIX:
            if (bytes > 0 && fseeko(f, (off_t)bytes, SEEK_CUR) != 0) w.ok = false;
            break;
        default: zero_fill(bytes); break;
        }
    }
    const long long total = ref_var_offset(R_NUM_VARIABLES, r);
    if (w.ok) w.ok = fflush(f) == 0 && ftruncate(fileno(f), (off_t)total) == 0;   // the hole up to the end
    const bool closed = std::fclose(f) == 0;
    if (!w.ok || !closed) {
        err_ = "DataIO: short write to " + path;
        return PD_ERR_FILE;
    }
    return PD_OK;
}

// DataIO::loadState (dataIO.cu:152-198) of a file in the reference's layout,
// into a handle made ready on the same scene: the counts come from
// DATA/sim_info.dat (num_pd_particle must match), the original positions must
// equal this handle's (to 1e-12 of their magnitude, after the scaleFactor
// division) and every particle's bonds must be among its initial bonds.  Read:
// positions (divided by scaleFactor) and velocities with their backups,
// stretch limits, bond lists with their tops and backup tops, the CG solution
// (the next solve's initial guess) and savedFrame; pd_time_step and clockScale
// from sim_info.dat.  The step counter becomes `timestep` (the reference keeps
// its step counter out of the file).  Not read: the system matrix and vector
// (rebuilt every step), SPH and cell arrays.
pd_status Engine::dataio_load_state_reference(size_t timestep)
{
    if (!ready_) {
        err_ = "DataIO: make_ready has not run (load a state into a handle made ready on the same scene)";
        return PD_ERR_NOT_READY;
    }
    RefSimulationParameters r;
    {
        FILE* fi = std::fopen((std::string(run_.saving_path) + "/DATA/sim_info.dat").c_str(), "rb");
        Reader rd{fi};
        if (fi) {
            rd.get(r);
            std::fclose(fi);
        }
        if (!fi || !rd.ok) {
            err_ = "DataIO: DATA/sim_info.dat of the saved run is missing (it sizes the state's arrays)";
            return PD_ERR_FILE;
        }
    }
    if (r.num_pd_particle != n_ || r.num_sph_particle < 0 || r.num_cells < 0 || r.num_clists < 0 ||
        r.boundaryPlaneSize < 0) {
        err_ = "DataIO: inconsistent number of particles/cells with saved data";
        return PD_ERR_STATE;
    }
    const std::string path = ref_state_path(timestep);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err_ = "DataIO: cannot open " + path;
        return PD_ERR_FILE;
    }
    fseeko(f, 0, SEEK_END);
    const long long fsize = (long long)ftello(f);
    if (fsize != ref_var_offset(R_NUM_VARIABLES, r)) {
        std::fclose(f);
        err_ = "DataIO: " + path + " does not have the size sim_info.dat's counts give";
        return PD_ERR_FILE;
    }
    const size_t N = (size_t)n_;
    Reader rd{f};
    auto read_var = [&](int v, void* dst) {
        if (fseeko(f, (off_t)ref_var_offset(v, r), SEEK_SET) != 0) rd.ok = false;
        rd.bytes(dst, (size_t)ref_var_bytes(v, r));
    };
    size_t frame = 0;
    fseeko(f, 0, SEEK_SET);
    rd.get(frame);
    std::vector<double> pos(4 * N), pos_bk(4 * N), vel(4 * N), vel_bk(4 * N), opos(4 * N), sol(4 * N), st(N), ost(N),
        nst(N);
    std::vector<int32_t> act(N), top(N), topbk(N), blist((size_t)kRefMaxBonds * N);
    read_var(R_PD_ACTIVITY, act.data());
    read_var(R_PD_POSITION, pos.data());
    read_var(R_PD_POSITION_BACKUP, pos_bk.data());
    read_var(R_PD_VELOCITY, vel.data());
    read_var(R_PD_VELOCITY_BACKUP, vel_bk.data());
    read_var(R_PD_ORIGINAL_POSITION, opos.data());
    read_var(R_PD_ORIGINAL_STRETCH, ost.data());
    read_var(R_PD_STRETCH, st.data());
    read_var(R_PD_NEW_STRETCH, nst.data());
    read_var(R_PD_BOND_LIST, blist.data());
    read_var(R_PD_BOND_LIST_TOP, top.data());
    read_var(R_PD_BOND_LIST_TOP_BACKUP, topbk.data());
    read_var(R_PD_SYSTEM_SOLUTION, sol.data());
    std::fclose(f);
    if (!rd.ok) {
        err_ = "DataIO: " + path + " is truncated";
        return PD_ERR_FILE;
    }
    const double sf = r.scaleFactor != 0.0 ? r.scaleFactor : 1.0;
    for (size_t i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            pos[4 * i + k] /= sf;
            opos[4 * i + k] /= sf;
        }
    // the same scene: original positions and activity
    std::vector<double> X(4 * N);
    pd_status s = get(PD_VAR_ORIGINAL_POSITION, X.data(), X.size() * sizeof(double));
    if (s != PD_OK) return s;
    double xmax = 0.0, dmax = 0.0;
    for (size_t i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            xmax = std::max(xmax, std::fabs(X[4 * i + k]));
            dmax = std::max(dmax, std::fabs(X[4 * i + k] - opos[4 * i + k]));
        }
    bool same = dmax <= 1e-12 * std::max(xmax, 1e-300);
    for (size_t i = 0; i < N && same; ++i) same = (act[i] & 7) == (h_act_[i] & 7);
    if (!same) {
        err_ = "DataIO: " + path + " holds another scene (original positions or activity differ)";
        return PD_ERR_STATE;
    }
    // bond rows: the file's live bonds first, then those broken since the
    // backup, then the rest of the particle's initial bonds
    CK(cudaSetDevice(device_), "cudaSetDevice");
    CK(cudaStreamSynchronize(stream_), "state sync");
    const size_t slots = (size_t)std::max<long long>(total_slots_, 1);
    std::vector<int> rp(N + 1), col(slots), cnt(N), cbk(N);
    std::vector<float> id0;
    std::vector<float2> d0s;
    CK(cudaMemcpy(rp.data(), S_.row_ptr, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost), "download rp");
    CK(cudaMemcpy(col.data(), S_.col, sizeof(int) * slots, cudaMemcpyDeviceToHost), "download col");
    if (!fp64_) {
        id0.resize(slots);
        d0s.resize(slots);
        CK(cudaMemcpy(id0.data(), S_.inv_d0, sizeof(float) * slots, cudaMemcpyDeviceToHost), "download 1/d0");
        CK(cudaMemcpy(d0s.data(), S_.d0sq, sizeof(float2) * slots, cudaMemcpyDeviceToHost), "download d0^2");
    }
    std::vector<int> ncol(col);
    std::vector<float> nid0(id0);
    std::vector<float2> nd0s(d0s);
    std::vector<int> where;
    for (size_t o = 0; o < N; ++o) {
        const int sl = inv_[o], base = rp[sl], all = cnt_init_[sl];
        const int live = top[o] + 1, bk = topbk[o] + 1;
        if (live < 0 || bk < live || bk > all) {
            err_ = "DataIO: " + path + ": bond counts of particle " + std::to_string(o) + " do not fit its bonds";
            return PD_ERR_STATE;
        }
        // slot of each initial bond of this row, by the neighbour's caller index
        where.assign((size_t)all, 0);
        std::vector<char> taken((size_t)all, 0);
        int k = 0;
        for (int j = 0; j < bk; ++j) {
            const int q = blist[(size_t)j * N + o];
            int found = -1;
            for (int t = 0; t < all; ++t)
                if (!taken[t] && perm_[col[base + t]] == q) {
                    found = t;
                    break;
                }
            if (found < 0) {
                err_ = "DataIO: " + path + ": particle " + std::to_string(o) + " has a bond that is not among its "
                       "initial bonds";
                return PD_ERR_STATE;
            }
            taken[found] = 1;
            where[k++] = found;
        }
        for (int t = 0; t < all; ++t)
            if (!taken[t]) where[k++] = t;
        for (int j = 0; j < all; ++j) {
            ncol[base + j] = col[base + where[j]];
            if (!fp64_) {
                nid0[base + j] = id0[base + where[j]];
                nd0s[base + j] = d0s[base + where[j]];
            }
        }
        cnt[sl] = live;
        cbk[sl] = bk;
    }
    // slot-order arrays
    auto to_slots4 = [&](const std::vector<double>& a) {
        std::vector<dbl4> out(N);
        for (size_t sl = 0; sl < N; ++sl) {
            const double* p = &a[4 * (size_t)perm_[sl]];
            out[sl] = make_dbl4(p[0], p[1], p[2], 0.0);
        }
        return out;
    };
    auto to_slots1 = [&](const std::vector<double>& a) {
        std::vector<double> out(N);
        for (size_t sl = 0; sl < N; ++sl) out[sl] = a[(size_t)perm_[sl]];
        return out;
    };
    const std::vector<dbl4> x4 = to_slots4(pos), xb4 = to_slots4(pos_bk), v4 = to_slots4(vel), vb4 = to_slots4(vel_bk),
                            s4 = to_slots4(sol);
    const std::vector<double> st1 = to_slots1(st), ost1 = to_slots1(ost), nst1 = to_slots1(nst);
    if (N) {
        CK(cudaMemcpy(S_.x64, x4.data(), sizeof(dbl4) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.x64_bk, xb4.data(), sizeof(dbl4) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.v64, v4.data(), sizeof(dbl4) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.v64_bk, vb4.data(), sizeof(dbl4) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.st, st1.data(), sizeof(double) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.ost, ost1.data(), sizeof(double) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.nst, nst1.data(), sizeof(double) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.cnt, cnt.data(), sizeof(int) * N, cudaMemcpyHostToDevice), "upload state");
        CK(cudaMemcpy(S_.cnt_bk, cbk.data(), sizeof(int) * N, cudaMemcpyHostToDevice), "upload state");
        if (fp64_) {
            CK(cudaMemcpy(S_.sol, s4.data(), sizeof(dbl4) * N, cudaMemcpyHostToDevice), "upload state");
        } else {
            std::vector<float4> sf4(N);
            for (size_t i = 0; i < N; ++i)
                sf4[i] = make_float4((float)s4[i].x, (float)s4[i].y, (float)s4[i].z, 0.f);
            CK(cudaMemcpy(S_.sol, sf4.data(), sizeof(float4) * N, cudaMemcpyHostToDevice), "upload state");
        }
    }
    if (total_slots_ > 0) {
        CK(cudaMemcpy(S_.col, ncol.data(), sizeof(int) * (size_t)total_slots_, cudaMemcpyHostToDevice), "upload bonds");
        if (!fp64_) {
            CK(cudaMemcpy(S_.inv_d0, nid0.data(), sizeof(float) * (size_t)total_slots_, cudaMemcpyHostToDevice),
               "upload bonds");
            CK(cudaMemcpy(S_.d0sq, nd0s.data(), sizeof(float2) * (size_t)total_slots_, cudaMemcpyHostToDevice),
               "upload bonds");
        }
    }
    saved_frame_ = frame;
    step_ = (int)timestep;
    substep_ = 0;
    ticks_ = r.pd_time_step > 0 ? r.pd_time_step : sim_.pd_time_step;
    clock_scale_ = r.clockScale;
    // the file holds no simulated time: step x the saved time step (exact
    // unless the adaptive scheme changed the step earlier in the run)
    sim_time_ = (double)step_ * ticks_ * opt_.time_step_base;
    cg_converged_ = true;
    predicted_iters_ = 0;
    hist_reset();
    retries_ = 0;
    // the rows now hold the file's order: the tuned SpMV shape's slot order is
    // laid out again from the build order
    lay_g_ = lay_u_ = 1;
    if (!L_.lattice && !L_.tiled) relayout_bonds(L_.lanes, L_.unroll);
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

pd_status pd_dataio_save_state_reference(pd_handle* h, size_t timestep)
{
    if (!h || !h->eng) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->dataio_save_state_reference(timestep);
}

pd_status pd_dataio_load_state_reference(pd_handle* h, size_t timestep)
{
    if (!h || !h->eng) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->dataio_load_state_reference(timestep);
}

pd_status pd_dataio_load_state(pd_handle* h, size_t timestep)
{
    if (!h || !h->eng) return PD_ERR_INVALID_ARGUMENT;
    return h->eng->dataio_load_state(timestep);
}

}  // extern "C"
