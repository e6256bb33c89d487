// dem_engine.cu -- host side of the GB300 DEM engine and its C ABI.
//
// Engine::init restates CudaDemSolver::initialize (src/cuda_backend_cuda.cu:
// 302-381, component ordering of uploadComponents :121-190); forces() the
// pipeline of computeForces (:383-524); the leapfrog entry points :526-543;
// the checkpoint the DMHIST2 format of :545-822.  runSteps() drives the
// integration loop of src/cuda_simulation_integrator.cpp:245-446 with the
// host MBD step of src/dyneq.cpp:97-130.
#include "../../include/dem_gb300.h"
#include "dem_adjoint.cuh"
#include "dem_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <unordered_set>
#include <vector>

namespace demgb {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

struct DemError : std::runtime_error {
    int code;
    DemError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

static void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw DemError(DEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

class DeviceArena {
public:
    ~DeviceArena() { release(); }
    template <typename T> T* alloc(size_t count, const char* what)
    {
        if (count == 0) count = 1;
        void* p = nullptr;
        check(cudaMalloc(&p, count * sizeof(T)), what);
        ptrs_.push_back(p);
        bytes_ += count * sizeof(T);
        return static_cast<T*>(p);
    }
    template <typename T> T* upload(const T* src, size_t count, const char* what, cudaStream_t s)
    {
        T* d = alloc<T>(count, what);
        if (count && src) check(cudaMemcpyAsync(d, src, count * sizeof(T), cudaMemcpyHostToDevice, s), what);
        return d;
    }
    void release()
    {
        for (void* p : ptrs_) cudaFree(p);
        ptrs_.clear();
        bytes_ = 0;
    }
    size_t bytes() const { return bytes_; }

private:
    std::vector<void*> ptrs_;
    size_t bytes_ = 0;
};

// Contact items up to which the PT law runs one warp per item.
constexpr int kDefaultPtWarpItems = 3072;
// Sweep blocks per SM: the sweep leaves warp slots to the PT and rotational
// branches that run beside it (0 would launch one thread per component).
// Scenes of up to kSmallScene components leave more room (their PT and
// rotational branches are short chains that must not wait for slots);
// larger scenes are throughput bound and give the sweep and the gathers
// more of each SM, grid-stride over three times the sweep's residency of 8
// blocks (scenes without triangles too: one thread per component took the
// 256-scene batch's step to 2.93 ms against 2.56 with 16 and 24 per SM).
// Measured on GB300 (200k- and 2M-sphere scenes, the 5.46M-sphere batch);
// the autotuner refines them per scene.
constexpr int kSmallScene = 500000;
constexpr int kSweepBlocksSmall = 3, kSweepBlocksLarge = 24;
// The gathers and the particle law, likewise (blocks of 256 per SM).  With
// the sweep at 8 resident blocks the gathers want fewer blocks than before
// (8 -> 4 on the drum 1.035 -> 1.031 ms and on the 256-scene batch 2.55 ->
// 2.53; 2 -> 3 on C1 0.1933 -> 0.1925).
constexpr int kGatherBlocksSmall = 3, kGatherBlocksLarge = 4;
constexpr int kDefaultPpBlocksPerSm = 16;

static MatF to_float(const MatC& c)
{
    return MatF{(float)c.kN, (float)c.kS, (float)c.logN, (float)c.logS, (float)c.denN, (float)c.denS, (float)c.mu,
                (float)c.muT, (float)c.muR, (float)c.beta, (float)c.coh, (float)c.dt};
}

static MatC make_mat(const dem_mech& m, double dt)
{
    MatC c;
    c.kN = m.kN;
    c.kS = 2.0 * m.kN / 7.0;
    c.logN = std::log(m.epsN);
    c.logS = std::log(m.epsS);
    c.denN = kPi * kPi + c.logN * c.logN;
    c.denS = kPi * kPi + c.logS * c.logS;
    c.mu = m.mu; c.muT = m.muT; c.muR = m.muR; c.beta = m.beta; c.coh = m.cohesion;
    c.dt = dt;
    return c;
}

class Engine {
public:
    ~Engine()
    {
        for (cudaGraphExec_t g : graphs_)
            if (g) cudaGraphExecDestroy(g);
        adj_release_graphs();
        for (auto* e : ev_) if (e) cudaEventDestroy(e);
        for (auto* e : fork_ev_) if (e) cudaEventDestroy(e);
        if (body_ready_) cudaEventDestroy(body_ready_);
        for (auto* e : adj_ev_) if (e) cudaEventDestroy(e);
        arena_.release();
        if (pinned_) cudaFreeHost(pinned_);
        if (diag_pin_) cudaFreeHost(diag_pin_);
        for (auto* b : branch_) if (b) cudaStreamDestroy(b);
        if (stream_) cudaStreamDestroy(stream_);
    }

    // ---------------------------------------------------------------- init
    void init(const dem_scene* scenes, int nscenes, const dem_options* opt)
    {
        if (initialized_) throw DemError(DEM_ERR_STATE, "CUDA DEM solver already initialized");
        if (!scenes || nscenes <= 0) throw DemError(DEM_ERR_INVALID, "no scenes");
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0)
            throw DemError(DEM_ERR_NO_DEVICE, "no CUDA device is available");
        dem_options o;
        dem_default_options(&o);
        if (opt) o = *opt;
        if (o.cell_factor < 2.0) throw DemError(DEM_ERR_INVALID, "cell_factor must be >= 2");
        precision_ = o.precision;
        pt_fp32_ = (o.precision == DEM_PRECISION_MIXED) && o.pt_fp32;
        cell_factor_ = o.cell_factor;
        block_ = o.block_size > 0 ? o.block_size : 128;
        check(cudaFree(nullptr), "initialize CUDA context");
        int dev = 0;
        check(cudaGetDevice(&dev), "cudaGetDevice");
        check(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, dev), "SM count");
        size_t total_mem = 0;
        check(cudaMemGetInfo(&free_before_, &total_mem), "cudaMemGetInfo");
        check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto*& e : ev_) check(cudaEventCreate(&e), "cudaEventCreate");
        {
            // The triangle/PT branch and the rotational branch carry the
            // critical paths (PT on few-item scenes, the FP64 advance on
            // large ones): their blocks are scheduled first as SM slots free.
            int lo = 0, hi = 0;
            check(cudaDeviceGetStreamPriorityRange(&lo, &hi), "stream priorities");
            const int prio[3] = {lo, hi, hi};
            for (int b = 0; b < 3; ++b)
                check(cudaStreamCreateWithPriority(&branch_[b], cudaStreamNonBlocking, prio[b]), "cudaStreamCreate");
        }
        for (auto*& e : fork_ev_) check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        check(cudaEventCreateWithFlags(&body_ready_, cudaEventDisableTiming), "cudaEventCreate");
        for (auto*& e : adj_ev_) check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");

        S_ = nscenes;
        dt_ = scenes[0].dt;
        // ---- concatenate scenes on the host
        std::vector<int> oid, ost, oscene;
        std::vector<double> om, orad, oin, opos, ovel, oomg, oq;
        std::vector<int> cown, cid;
        std::vector<double> crad, cbody;
        std::vector<double> wo, wn;
        std::vector<double> bmass, bc, bq, bv, bw, bin;
        std::vector<int> bstate, bscene;
        std::vector<int> tbody, tscene;
        std::vector<double> tloc;
        std::vector<SceneC> sc(nscenes);
        bool any_clump = false, any_ug = false;
        std::vector<double> scene_rmax(nscenes, 0.0);
        nbs_ = 0;
        for (int s = 0; s < nscenes; ++s) {
            const dem_scene& x = scenes[s];
            if (x.n_owners <= 0) throw DemError(DEM_ERR_INVALID, "CUDA DEM solver requires particles");
            if (x.dt != dt_) throw DemError(DEM_ERR_INVALID, "all scenes of a batch must share dt");
            if (!x.owner_id || !x.owner_status || !x.owner_mass || !x.owner_radius || !x.owner_inertia ||
                !x.owner_pos || !x.owner_vel || !x.owner_omega || !x.owner_quat)
                throw DemError(DEM_ERR_INVALID, "scene owner arrays must not be NULL");
            std::unordered_set<int> ids;
            ids.reserve((size_t)x.n_owners);
            for (int i = 0; i < x.n_owners; ++i)
                if (!ids.insert(x.owner_id[i]).second)
                    throw DemError(DEM_ERR_INVALID, "duplicate particle ID " + std::to_string(x.owner_id[i]) +
                                                        "; contact history requires stable unique particle IDs");
            const int obase = (int)oid.size();
            for (int i = 0; i < x.n_owners; ++i) {
                oid.push_back(x.owner_id[i]); ost.push_back(x.owner_status[i]); oscene.push_back(s);
                om.push_back(x.owner_mass[i]); orad.push_back(x.owner_radius[i]);
                for (int a = 0; a < 3; ++a) {
                    oin.push_back(x.owner_inertia[3 * i + a]); opos.push_back(x.owner_pos[3 * i + a]);
                    ovel.push_back(x.owner_vel[3 * i + a]); oomg.push_back(x.owner_omega[3 * i + a]);
                }
                for (int a = 0; a < 4; ++a) oq.push_back(x.owner_quat[4 * i + a]);
            }
            // components: uploadComponents ordering (owner, component id)
            const int nc = x.n_components > 0 ? x.n_components : x.n_owners;
            std::vector<int> order(nc);
            std::iota(order.begin(), order.end(), 0);
            auto own = [&](int c) { return x.n_components > 0 ? x.comp_owner[c] : c; };
            auto idf = [&](int c) { return x.n_components > 0 ? x.comp_id[c] : x.owner_id[c]; };
            if (x.n_components > 0) {
                any_clump = true;
                std::sort(order.begin(), order.end(), [&](int a, int b) {
                    if (own(a) != own(b)) return own(a) < own(b);
                    return idf(a) < idf(b);
                });
            }
            std::vector<int> per_owner(x.n_owners, 0);
            for (int k = 0; k < nc; ++k) {
                const int c = order[k];
                const int ow = own(c);
                const double r = x.n_components > 0 ? x.comp_radius[c] : x.owner_radius[c];
                if (ow < 0 || ow >= x.n_owners || idf(c) < 0 || !std::isfinite(r) || r <= 0.0)
                    throw DemError(DEM_ERR_INVALID, "invalid native clump component topology");
                per_owner[ow]++;
                cown.push_back(obase + ow);
                cid.push_back(idf(c));
                crad.push_back(r);
                for (int a = 0; a < 3; ++a) cbody.push_back(x.n_components > 0 ? x.comp_offset[3 * c + a] : 0.0);
                max_radius_ = std::max(max_radius_, r);
                scene_rmax[s] = std::max(scene_rmax[s], r);
                comp_owner_ids_.push_back(x.owner_id[ow]);
            }
            for (int i = 0; i < x.n_owners; ++i)
                if (per_owner[i] < 1 || per_owner[i] > 8)
                    throw DemError(DEM_ERR_INVALID, "each CUDA owner requires 1 to 8 components");
            SceneC& S = sc[s];
            S.pp = make_mat(x.pp, x.dt); S.pt = make_mat(x.pt, x.dt); S.pw = make_mat(x.pw, x.dt);
            S.ppf = to_float(S.pp); S.ptf = to_float(S.pt); S.pwf = to_float(S.pw);
            S.mesh = cell_factor_ * scene_rmax[s];
            if (!(S.mesh > 0.0)) throw DemError(DEM_ERR_INVALID, "invalid mesh size");
            S.inv_mesh = 1.0 / S.mesh;
            S.pad = scene_rmax[s];
            S.mesh_f = (float)S.mesh;
            S.margin_f = (float)(1.0e-5 * S.mesh);
            S.inv_mesh_f = (float)S.inv_mesh;
            set_skin(S);
            for (int a = 0; a < 3; ++a) S.g[a] = x.gravity[a];
            S.grav = x.gravity_enabled ? 1 : 0;
            S.wall_begin = (int)wo.size() / 3;
            S.wall_count = x.n_walls > 0 ? x.n_walls : 0;
            for (int w = 0; w < S.wall_count; ++w)
                for (int a = 0; a < 3; ++a) { wo.push_back(x.wall_origin[3 * w + a]); wn.push_back(x.wall_normal[3 * w + a]); }
            S.body_begin = (int)bmass.size();
            S.body_count = x.n_bodies > 0 ? x.n_bodies : 0;
            nbs_ = std::max(nbs_, S.body_count);
            for (int b = 0; b < S.body_count; ++b) {
                bmass.push_back(x.body_mass[b]);
                for (int a = 0; a < 3; ++a) { bc.push_back(x.body_center[3 * b + a]); bv.push_back(x.body_vel[3 * b + a]); bw.push_back(x.body_omega[3 * b + a]); }
                for (int a = 0; a < 4; ++a) bq.push_back(x.body_quat[4 * b + a]);
                for (int a = 0; a < 9; ++a) bin.push_back(x.body_inertia[9 * b + a]);
                bstate.push_back(x.body_state ? x.body_state[b] : 0);
                bscene.push_back(s);
            }
            if (S.body_count > 0 && x.n_triangles > 0) {
                for (int t = 0; t < x.n_triangles; ++t) {
                    const int b = x.tri_body[t];
                    if (b < 0 || b >= S.body_count) throw DemError(DEM_ERR_INVALID, "triangle body index out of range");
                    tbody.push_back(S.body_begin + b);
                    tscene.push_back(s);
                    for (int a = 0; a < 15; ++a) tloc.push_back(x.tri_local[15 * t + a]);
                }
            }
            if (x.universal_gravity_enabled) any_ug = true;
            keep_bp_ = keep_bp_ || x.keep_body_particle;
            keep_bd_ = keep_bd_ || x.keep_body_detail;
            grav_.push_back(x.gravity_enabled ? 1 : 0);
            gvec_.push_back({x.gravity[0], x.gravity[1], x.gravity[2]});
        }
        n_ = (int)oid.size();
        // the contact list and the history slots hold kPSlots entries per
        // component and are indexed by int
        if (cown.size() > (size_t)INT_MAX / kPSlots)
            throw DemError(DEM_ERR_CAPACITY, "more than " + std::to_string(INT_MAX / kPSlots) +
                                                 " components: per-component contact slots exceed the int index range");
        nc_ = (int)cown.size();
        nw_ = (int)wo.size() / 3;
        nb_ = (int)bmass.size();
        nt_ = (int)tbody.size();
        sphere_ = !any_clump;
        owner_ids_ = oid;
        comp_ids_ = cid;
        comp_radius_ = crad;
        comp_body_ = cbody;
        body_mass_ = bmass; body_inertia_ = bin; body_state_ = bstate; body_scene_ = bscene;
        hbc_ = bc; hbq_ = bq; hbv_ = bv; hbw_ = bw;
        mesh_ = cell_factor_ * max_radius_;
        if (!(mesh_ > 0.0)) throw DemError(DEM_ERR_INVALID, "invalid mesh size");
        cudaStream_t s = stream_;

        // ---- owners
        O_.n = n_;
        auto col = [&](const std::vector<double>& v, int stride, int a) {
            std::vector<double> out(n_);
            for (int i = 0; i < n_; ++i) out[i] = v[(size_t)stride * i + a];
            return out;
        };
        auto upd = [&](const std::vector<double>& v, const char* w) { return arena_.upload(v.data(), v.size(), w, s); };
        std::vector<std::vector<double>> cols;
        for (int a = 0; a < 3; ++a) cols.push_back(col(opos, 3, a));
        for (int a = 0; a < 3; ++a) cols.push_back(col(ovel, 3, a));
        for (int a = 0; a < 3; ++a) cols.push_back(col(oomg, 3, a));
        for (int a = 0; a < 4; ++a) cols.push_back(col(oq, 4, a));
        for (int a = 0; a < 3; ++a) cols.push_back(col(oin, 3, a));
        O_.px = upd(cols[0], "px"); O_.py = upd(cols[1], "py"); O_.pz = upd(cols[2], "pz");
        O_.vx = upd(cols[3], "vx"); O_.vy = upd(cols[4], "vy"); O_.vz = upd(cols[5], "vz");
        O_.wx = upd(cols[6], "wx"); O_.wy = upd(cols[7], "wy"); O_.wz = upd(cols[8], "wz");
        O_.qw = upd(cols[9], "qw"); O_.qx = upd(cols[10], "qx"); O_.qy = upd(cols[11], "qy"); O_.qz = upd(cols[12], "qz");
        O_.ix = upd(cols[13], "ix"); O_.iy = upd(cols[14], "iy"); O_.iz = upd(cols[15], "iz");
        O_.mass = upd(om, "mass"); O_.radius = upd(orad, "radius");
        {
            std::vector<double> inv(n_);
            for (int i = 0; i < n_; ++i) inv[i] = 1.0 / om[i];
            O_.inv_mass = upd(inv, "inverse mass");
            std::vector<double> mg(3 * (size_t)n_, 0.0);
            for (int i = 0; i < n_; ++i) {
                const SceneC& S = sc[oscene[i]];
                if (S.grav)
                    for (int a = 0; a < 3; ++a) mg[3 * (size_t)i + a] = om[i] * S.g[a];
            }
            O_.mg = upd(mg, "field force");
            for (int a = 0; a < 3; ++a) {
                for (int i = 0; i < n_; ++i) inv[i] = 1.0 / oin[3 * (size_t)i + a];
                (a == 0 ? O_.inv_ix : (a == 1 ? O_.inv_iy : O_.inv_iz)) = upd(inv, "inverse inertia");
            }
            std::vector<unsigned char> iso(n_);
            std::vector<float> iif(n_);
            for (int i = 0; i < n_; ++i) {
                const double* I = &oin[3 * (size_t)i];
                iso[i] = (I[0] == I[1] && I[1] == I[2]) ? 1 : 0;
                iif[i] = (float)(1.0 / I[0]);
            }
            O_.iso = arena_.upload(iso.data(), iso.size(), "isotropic flags", s);
            oin_host_ = oin;
            O_.inv_i_f = arena_.upload(iif.data(), iif.size(), "fp32 inverse inertia", s);
        }
        double** zeros[] = {&O_.ax, &O_.ay, &O_.az, &O_.awx, &O_.awy, &O_.awz, &O_.vhx, &O_.vhy, &O_.vhz,
                            &O_.whx, &O_.why, &O_.whz, &O_.hqw, &O_.hqx, &O_.hqy, &O_.hqz};
        for (double** z : zeros) {
            *z = arena_.alloc<double>(n_, "owner state");
            check(cudaMemsetAsync(*z, 0, sizeof(double) * n_, s), "clear owner state");
        }
        O_.id = arena_.upload(oid.data(), oid.size(), "id", s);
        O_.status = arena_.upload(ost.data(), ost.size(), "status", s);
        O_.scene = arena_.upload(oscene.data(), oscene.size(), "scene", s);
        if (any_ug) {
            O_.ugx = arena_.alloc<double>(n_, "ug"); O_.ugy = arena_.alloc<double>(n_, "ug"); O_.ugz = arena_.alloc<double>(n_, "ug");
        }

        // ---- components
        C_.n = nc_;
        C_.sphere = sphere_ ? 1 : 0;
        C_.owner = arena_.upload(cown.data(), cown.size(), "comp owner", s);
        C_.cid = arena_.upload(cid.data(), cid.size(), "comp id", s);
        C_.radius = arena_.upload(crad.data(), crad.size(), "comp radius", s);
        if (sphere_) {
            C_.x = O_.px; C_.y = O_.py; C_.z = O_.pz; C_.vx = O_.vx; C_.vy = O_.vy; C_.vz = O_.vz;
            C_.vhx = O_.vhx; C_.vhy = O_.vhy; C_.vhz = O_.vhz;
        } else {
            std::vector<int> ostart(n_ + 1, 0);
            for (int c = 0; c < nc_; ++c) ostart[cown[c] + 1]++;
            for (int i = 0; i < n_; ++i) ostart[i + 1] += ostart[i];
            C_.ostart = arena_.upload(ostart.data(), ostart.size(), "ostart", s);
            std::vector<double> bx(nc_), by(nc_), bz(nc_);
            for (int c = 0; c < nc_; ++c) { bx[c] = cbody[3 * c]; by[c] = cbody[3 * c + 1]; bz[c] = cbody[3 * c + 2]; }
            C_.bx = upd(bx, "bx"); C_.by = upd(by, "by"); C_.bz = upd(bz, "bz");
            double** cw[] = {&C_.x, &C_.y, &C_.z, &C_.vx, &C_.vy, &C_.vz, &C_.vhx, &C_.vhy, &C_.vhz, &C_.ox, &C_.oy, &C_.oz};
            for (double** z : cw) *z = arena_.alloc<double>(nc_, "component world state");
        }

        d_sc_ = arena_.upload(sc.data(), sc.size(), "scene constants", s);
        G_.sc = d_sc_;

        // ---- grid
        long long cap = o.max_cells > 0 ? o.max_cells : std::max<long long>(16LL * nc_, 1LL << 22);
        cap = std::min<long long>(cap, (1LL << 31) - 64);
        G_.capacity = (int)cap;
        G_.nscenes = S_;
        G_.ckey = arena_.alloc<uint64_t>(nc_, "ckey");
        G_.clin = arena_.alloc<int>(nc_, "clin");
        G_.crank = arena_.alloc<int>(nc_, "crank");
        G_.cell_count = arena_.alloc<int>(cap + 1, "cell count");
        check(cudaMemsetAsync(G_.cell_count, 0, sizeof(int) * (cap + 1), s), "clear cell count");
        G_.cell_start = arena_.alloc<int>(cap + 2, "cell start");
        G_.sorted_id = arena_.alloc<int>(nc_, "sorted id");
        G_.pos_of = arena_.alloc<int>(nc_, "pos of");
        G_.sorted_tmp = arena_.alloc<int>(nc_, "sorted scratch");
        G_.sorted_key = arena_.alloc<uint64_t>(nc_, "sorted key");
        std::vector<int> box(6 * S_);
        for (int q = 0; q < S_; ++q) { box[6 * q] = box[6 * q + 1] = box[6 * q + 2] = INT_MAX; box[6 * q + 3] = box[6 * q + 4] = box[6 * q + 5] = INT_MIN; }
        G_.scene_box = arena_.upload(box.data(), box.size(), "scene box", s);
        G_.scene_layout = arena_.alloc<int>(8 * S_, "scene layout");
        G_.total_cells = arena_.alloc<int>(1, "total cells");
        G_.nvalid = arena_.alloc<int>(1, "nvalid");
        G_.scan = alloc_scan(cap + 1, 4096, "cell scan");
        // Diagnostics block, one allocation so that one copy reads it back:
        // 16 counters, the error word, then the interval sums the reference
        // resets at every diagnostic read (regime counts, microstate sums,
        // native steps).
        diag_bytes_ = kDiagIntervalOff + sizeof(double) * ((size_t)nb_ * (kRegime + kMicro) + 1);
        diag_dev_ = arena_.alloc<char>(diag_bytes_, "diagnostics");
        check(cudaMemsetAsync(diag_dev_, 0, diag_bytes_, s), "clear diagnostics");
        check(cudaMallocHost(&diag_pin_, diag_bytes_), "cudaMallocHost");
        G_.err = reinterpret_cast<unsigned*>(diag_dev_ + 64);

        // ---- records
        R_.pos = arena_.alloc<D4>(nc_, "rec pos");
        if (precision_ == DEM_PRECISION_MIXED) {
            R_.vf = arena_.alloc<float4>(nc_, "rec v"); R_.vmf = arena_.alloc<float4>(nc_, "rec vm");
            R_.wf = arena_.alloc<float4>(nc_, "rec w"); R_.wmf = arena_.alloc<float4>(nc_, "rec wm");
        } else {
            R_.v = arena_.alloc<D4>(nc_, "rec v"); R_.vm = arena_.alloc<D4>(nc_, "rec vm");
            R_.w = arena_.alloc<D4>(nc_, "rec w"); R_.wm = arena_.alloc<D4>(nc_, "rec wm");
        }
        R_.off = sphere_ ? nullptr : arena_.alloc<D4>(nc_, "rec off");
        R_.meta = arena_.alloc<int4>(nc_, "rec meta"); R_.cell = arena_.alloc<int4>(nc_, "rec cell");
        R_.relf = arena_.alloc<float4>(nc_, "rec relf");

        // ---- walls, bodies, triangles
        W_.count = (int)(wo.size() / 3);
        W_.o = upd(wo, "wall origin"); W_.n = upd(wn, "wall normal");
        {
            std::vector<float4> pl(wo.size() / 3);
            for (size_t k = 0; k < pl.size(); ++k) {
                const double nd = wn[3 * k] * wo[3 * k] + wn[3 * k + 1] * wo[3 * k + 1] + wn[3 * k + 2] * wo[3 * k + 2];
                pl[k] = make_float4((float)wn[3 * k], (float)wn[3 * k + 1], (float)wn[3 * k + 2], (float)nd);
            }
            W_.plane = arena_.upload(pl.data(), pl.size(), "wall planes", s);
        }
        B_.nb = nb_;
        {
            // c, q, v, w of all bodies in one block, in the pinned staging
            // layout, so a step's body state moves in one copy
            std::vector<double> st;
            st.insert(st.end(), bc.begin(), bc.end());
            st.insert(st.end(), bq.begin(), bq.end());
            st.insert(st.end(), bv.begin(), bv.end());
            st.insert(st.end(), bw.begin(), bw.end());
            st.resize(13 * (size_t)std::max(nb_, 1), 0.0);
            B_.c = arena_.upload(st.data(), st.size(), "body state", s);
            const size_t m = (size_t)std::max(nb_, 1);
            B_.q = B_.c + 3 * m; B_.v = B_.c + 7 * m; B_.w = B_.c + 10 * m;
        }
        B_.scene = arena_.upload(bscene.data(), bscene.size(), "body scene", s);
        T_.nt = nt_;
        if (nt_ > 0) {
            T_.body = arena_.upload(tbody.data(), tbody.size(), "tri body", s);
            T_.scene = arena_.upload(tscene.data(), tscene.size(), "tri scene", s);
            T_.local = upd(tloc, "tri local");
            T_.world = arena_.alloc<double>(16 * (size_t)nt_, "tri world");
            T_.trange = arena_.alloc<int>(6 * (size_t)nt_, "tri cell range");
            T_.tf = arena_.alloc<float4>(2 * (size_t)nt_, "tri fp32 planes");
            // rotation-invariant bound of the cells a padded triangle box covers
            long long tcap = 0;
            for (int t = 0; t < nt_; ++t) {
                const double* L = &tloc[15 * (size_t)t];
                double cx = 0, cy = 0, cz = 0;
                for (int k = 0; k < 4; ++k) { cx += L[3 * k]; cy += L[3 * k + 1]; cz += L[3 * k + 2]; }
                cx /= 4; cy /= 4; cz /= 4;
                double rho = 0;
                for (int k = 0; k < 4; ++k)
                    rho = std::max(rho, std::sqrt((L[3 * k] - cx) * (L[3 * k] - cx) + (L[3 * k + 1] - cy) * (L[3 * k + 1] - cy) +
                                                  (L[3 * k + 2] - cz) * (L[3 * k + 2] - cz)));
                const SceneC& St = sc[tscene[t]];
                const long long per = (long long)std::floor((2 * rho + 2 * St.pad) / St.mesh) + 2;
                tcap += per * per * per;
            }
            tcap = std::min<long long>(tcap + 1024, (1LL << 31) - 64);
            T_.capacity = (int)tcap;
            T_.ttri = arena_.alloc<int>(tcap, "tri grid ids");
            T_.ttri_tmp = arena_.alloc<int>(tcap, "tri grid scratch ids");
            T_.tlin_tmp = arena_.alloc<int>(tcap, "tri grid scratch cells");
            T_.tcell_count = arena_.alloc<int>(cap + 1, "tri cell count");
            T_.tcell_cursor = arena_.alloc<int>(cap + 1, "tri cell cursor");
            T_.tcell_start = arena_.alloc<int>(cap + 2, "tri cell start");
            check(cudaMemsetAsync(T_.tcell_count, 0, sizeof(int) * (cap + 1), s), "clear");
            check(cudaMemsetAsync(T_.tcell_cursor, 0, sizeof(int) * (cap + 1), s), "clear");
            T_.scan = alloc_scan(cap + 1, 4096, "triangle scan");
        }

        // ---- counters
        int* cnt = reinterpret_cast<int*>(diag_dev_);
        K_.pcontacts = cnt; K_.pover = cnt + 1; K_.bover = cnt + 2; K_.phigh = cnt + 3; K_.bhigh = cnt + 4;
        K_.tgover = cnt + 5; K_.ct_total = cnt + 6; K_.step = cnt + 8;
        K_.pt_ctotal = cnt + 9;
        K_.wl_total = cnt + 10;
        K_.pt_warp_items = kDefaultPtWarpItems;
        // without triangles no PT branch needs room beside the sweep
        K_.sweep_bps = nt_ > 0 && nc_ <= kSmallScene ? kSweepBlocksSmall : kSweepBlocksLarge;
        K_.gather_bps = nc_ <= kSmallScene ? kGatherBlocksSmall : kGatherBlocksLarge;
        K_.pp_bps = kDefaultPpBlocksPerSm;
        // neighbour lists (set_launch 3 turns them off)
        K_.nl_on = 1;
        K_.nl_flag = arena_.alloc<int>(4, "neighbour lists");
        check(cudaMemsetAsync(K_.nl_flag, 0, 4 * sizeof(int), s), "neighbour lists");
        K_.nl_hot = arena_.alloc<int>((size_t)G_.capacity, "neighbour lists");
        check(cudaMemsetAsync(K_.nl_hot, 0xff, sizeof(int) * (size_t)G_.capacity, s), "neighbour lists");
        K_.nl_limit = std::max(64, nc_ / 64);
        K_.nl_cnt = arena_.alloc<int>(nc_, "neighbour lists");
        K_.nl_idx = arena_.alloc<int>((size_t)nc_ * kNL, "neighbour lists");
        K_.nl_xref = arena_.alloc<double>(3 * (size_t)nc_, "neighbour lists");
        // no list yet: counts 0, build positions far away (about 1.4e306 m)
        check(cudaMemsetAsync(K_.nl_cnt, 0, sizeof(int) * nc_, s), "neighbour lists");
        check(cudaMemsetAsync(K_.nl_xref, 0x7f, sizeof(double) * 3 * (size_t)nc_, s), "neighbour lists");
        nl_request_rebuild();

        // ---- scene constants
        scenes_h_ = sc;

        // ---- history and contacts
        if (precision_ == DEM_PRECISION_MIXED) {
            if (pt_fp32_) alloc_state<float, float>(hp32_, hw32_, hb32_, ct32_);
            else alloc_state<float, double>(hp32_, hw32_, hb64_, ct32_);
        } else {
            alloc_state<double, double>(hp64_, hw64_, hb64_, ct64_);
        }

        // ---- body reduction
        if (nb_ > 0) {
            BO_.groups = std::max(1, std::min(sm_count_ * 16, (nc_ + 1023) / 1024));
            BO_.partial = arena_.alloc<double>((size_t)nb_ * BO_.groups * kBodyFieldCount, "body partial");
            BO_.result = arena_.alloc<double>((size_t)nb_ * kBodyFieldCount, "body result");
            check(cudaMemsetAsync(BO_.result, 0, sizeof(double) * nb_ * kBodyFieldCount, s), "clear");
            BO_.reg_int = reinterpret_cast<unsigned long long*>(diag_dev_ + kDiagIntervalOff);
            BO_.micro_int = reinterpret_cast<double*>(BO_.reg_int + (size_t)nb_ * kRegime);
            BO_.native_steps = reinterpret_cast<unsigned long long*>(BO_.micro_int + (size_t)nb_ * kMicro);
        }
        // pinned staging: body state (13 doubles/body) + body results
        pinned_bytes_ = sizeof(double) * ((size_t)13 * std::max(nb_, 1) + (size_t)kBodyFieldCount * std::max(nb_, 1) + 64);
        check(cudaMallocHost(&pinned_, pinned_bytes_), "cudaMallocHost");
        // host MBD state
        hbhv_.assign(3 * nb_, 0.0); hbhw_.assign(3 * nb_, 0.0); hbhq_.assign(4 * nb_, 0.0); hbhdq_.assign(4 * nb_, 0.0);
        hbacc_.assign(3 * nb_, 0.0); hbdom_.assign(3 * nb_, 0.0); hbloads_.assign(6 * nb_, 0.0);
        if (nb_ > 0) launch_tri_transform(T_, B_, d_sc_, s);
        if (!sphere_) launch_update_components(C_, O_, s);
        check(cudaStreamSynchronize(s), "initialize");
        initialized_ = true;
    }

    template <typename H> void mk_hist(Hist<H>& h, int slots)
    {
        cudaStream_t s = stream_;
        const size_t n = (size_t)nc_ * slots;
        h.key = arena_.alloc<uint64_t>(n, "history keys");
        h.last = arena_.alloc<int>(n, "history last seen");
        h.val = arena_.alloc<H>(n * kHV, "history values");
        h.hw = arena_.alloc<int>(nc_, "history hw");
        h.nc = nc_;
        check(cudaMemsetAsync(h.key, 0, n * sizeof(uint64_t), s), "clear history keys");
        check(cudaMemsetAsync(h.last, 0xff, n * sizeof(int), s), "clear history age");
        check(cudaMemsetAsync(h.val, 0, n * kHV * sizeof(H), s), "clear history values");
        check(cudaMemsetAsync(h.hw, 0, nc_ * sizeof(int), s), "clear history hw");
    }

    template <typename T, typename TB> void alloc_state(Hist<T>& hp, Hist<T>& hw, Hist<TB>& hb, Contacts<T>& ct)
    {
        cudaStream_t s = stream_;
        mk_hist(hp, kPSlots);
        mk_hist(hw, kWSlots);
        mk_hist(hb, kBSlots);
        ct.capacity = nc_ * kPSlots;
        ct.ent = arena_.alloc<int4>((size_t)ct.capacity, "contact entries");
        ct.res = arena_.alloc<T>((size_t)ct.capacity * 6, "contact results");
        ct.off = arena_.alloc<int>(nc_, "contact offsets");
        ct.cnt = arena_.alloc<int>(nc_, "contact counts");
        check(cudaMemsetAsync(ct.cnt, 0, nc_ * sizeof(int), s), "clear");
        check(cudaMemsetAsync(ct.off, 0, nc_ * sizeof(int), s), "clear");
        ct.wres = arena_.alloc<double>((size_t)nc_ * 6, "wall results");
        ct.wflag = arena_.alloc<unsigned char>(nc_, "wall flags");
        ct.wlist = arena_.alloc<int2>(nc_, "wall candidates");
        check(cudaMemsetAsync(ct.wflag, 0, nc_, s), "clear");
        check(cudaMemsetAsync(ct.wres, 0, (size_t)nc_ * 6 * sizeof(double), s), "clear");
        ct.pt_index = arena_.alloc<int>(nc_, "pt index");
        check(cudaMemsetAsync(ct.pt_index, 0xff, nc_ * sizeof(int), s), "clear");
        ct.nbs = std::max(nbs_, 1);
        if (nb_ > 0 && nt_ > 0) {
            ct.pt_clist = arena_.alloc<int>(nc_, "pt contact list");
            ct.pt_ctotal_ptr = K_.pt_ctotal;
            ct.pt_scan = alloc_scan((size_t)nc_ + 1, kPtItemTile, "pt item scan");
            ct.pt_res = arena_.alloc<double>((size_t)nc_ * 6, "pt results");
            ct.pt_body = arena_.alloc<double>((size_t)nc_ * ct.nbs * kPtRecord, "pt body records");
            if (keep_bp_ || keep_bd_) ct.pt_out = arena_.alloc<double>((size_t)nc_ * ct.nbs * 25, "pt outputs");
        }
    }

    // Status words and control words of a single-pass scan over up to n items
    // in tiles of `tile` (zeroed: epoch 0, nothing published).
    ScanState alloc_scan(size_t n, int tile, const char* what)
    {
        ScanState st;
        st.max_tiles = (int)(n / tile + 2);
        st.status = arena_.alloc<unsigned long long>((size_t)st.max_tiles, what);
        st.ctl = arena_.alloc<unsigned>(4, what);
        check(cudaMemsetAsync(st.status, 0, sizeof(unsigned long long) * st.max_tiles, stream_), what);
        check(cudaMemsetAsync(st.ctl, 0, sizeof(unsigned) * 4, stream_), what);
        return st;
    }

    // ----------------------------------------------------------- pipeline
    // Work a force evaluation carries at its ends: the body-frame triangle
    // transform before it, the body-result download after the body
    // reduction (with the event the host waits on for the MBD step), and
    // the leapfrog finish (or finish + the position part of the next
    // advance) after the owner sum.
    // kHeadRest puts the previous step's rotational advance (the second part
    // of a split finish + advance) at the head, beside the particle grid;
    // kTailFinishPos ends with the first part.
    // kHeadAdvance opens the first step of a run with the advance itself,
    // split the same way (positions first, the rest on the branch); with
    // kHeadRest as well, the rest is k_advance_rest, for a run whose previous
    // call ended with kTailFinishVel (the half-step velocities alone, the
    // quaternion rate left to the next advance).
    enum : unsigned {
        kTailTransform = 1, kTailD2H = 2, kTailFinish = 4, kHeadRest = 8, kTailFinishPos = 16, kHeadAdvance = 32,
        kTailDiag = 64, kTailFinishVel = 128
    };

    template <typename T, typename TB>
    void enqueue_forces(double dt_eff, Hist<T>& hp, Hist<T>& hw, Hist<TB>& hb, Contacts<T>& ct, bool timed,
                        unsigned tail)
    {
        cudaStream_t s = stream_;
        int e = 0;
        auto mark = [&]() { if (timed && e < (int)ev_.size()) check(cudaEventRecord(ev_[e++], s), "event"); };
        auto contacts = [&](int stage, cudaStream_t on) {
            launch_contacts<T, TB>(C_, O_, G_, R_, d_sc_, W_, T_, B_, hp, hw, hb, ct, K_, dt_eff, block_, sm_count_, on,
                                   stage);
        };
        const bool walls = W_.count > 0, pt = nb_ > 0 && nt_ > 0;
        auto integrate = [&](cudaStream_t on) {
            if (tail & kTailFinishPos) launch_finish_advance_pos(O_, dt_, on);
            else if (tail & kTailFinish) launch_finish(O_, dt_, on);
            else if (tail & kTailFinishVel) launch_finish_vel(O_, dt_, on);
        };
        // the rotational advance on a branch only for spheres: with clumps the
        // component update reads the quaternions at once
        const bool head_rot = tail & (kHeadRest | kHeadAdvance);
        const bool rest_branch = head_rot && !timed && sphere_;
        auto rotational = [&](cudaStream_t on) {
            if (tail & kHeadRest) launch_advance_rest(O_, dt_, sm_count_, on);
            else launch_advance_rot(O_, dt_, sm_count_, on);
        };
        if (tail & kHeadAdvance) launch_advance_pos(O_, dt_, s);
        if (head_rot && !rest_branch) rotational(s);
        auto download = [&](cudaStream_t on) {
            if (!(tail & kTailD2H) || nb_ <= 0) return;
            check(cudaMemcpyAsync(pin_body_result(), BO_.result, sizeof(double) * nb_ * kBodyFieldCount,
                                  cudaMemcpyDeviceToHost, on), "download body result");
            // in a captured graph the record must be an event node of its own
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            check(cudaStreamIsCapturing(on, &cs), "capture status");
            check(cudaEventRecordWithFlags(body_ready_, on,
                                           cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u),
                  "body result event");
        };
        if ((tail & kTailTransform) && nb_ > 0 && (timed || !pt)) launch_tri_transform(T_, B_, d_sc_, s);
        if (timed) {
            // one stream, phase by phase, for the phase timers
            mark();
            launch_step_counter(K_, 1, s);
            if (!sphere_) launch_update_components(C_, O_, s);
            launch_grid_layout(C_, O_, G_, s);
            launch_grid_sort(C_, O_, G_, sm_count_, s);
            mark();
            if (pt) launch_tri_build(T_, B_, G_, K_.tgover, sm_count_, s);
            if (O_.ugx) launch_universal_gravity(O_, s);
            launch_gather_geom(C_, O_, G_, R_, sm_count_, K_.gather_bps, K_, s);
            launch_gather_vel<T>(C_, O_, G_, R_, dt_eff, sm_count_, K_.gather_bps, s);
            mark();
            for (int stage : {2, 1, 4, 8, 16}) {
                contacts(stage, s);
                mark();
            }
            launch_owner_sum<T>(C_, O_, d_sc_, ct, false, nullptr, nullptr, nullptr, nullptr, s);
            mark();
            if (nb_ > 0) launch_body_reduce<T>(R_, d_sc_, B_, ct, BO_, dt_eff > 0.0, s);
            launch_step_counter(K_, 0, s);
            mark();
            n_marks_ = e;
            download(s);
            integrate(s);
            if (tail & kTailDiag) enqueue_diag_download(s);
            return;
        }
        // Branches (a DAG when captured into the step graph):
        //   main: cell keys and layout, the sort, the geometry gather, the
        //     sweep, the particle law, the owner sum, the integrator;
        //   rotational: the previous step's rotational advance, then (after
        //     the sort) the velocity gather;
        //   walls: after the step counter and the rotational advance;
        //   triangles: transform, triangle grid (after the layout), PT (after
        //     the geometry gather and the rotational advance), body
        //     reduction, body-result download.
        // The particle law waits for the velocity gather, the owner sum for
        // walls and PT.  Each branch touches its own history array and result
        // buffers (the wall and body slots expire in their own probes).
        cudaStream_t bw = branch_[0], bt = branch_[1], br = branch_[2];
        auto link = [&](cudaStream_t from, cudaStream_t to, int ev) {
            check(cudaEventRecord(fork_ev_[ev], from), "fork event");
            check(cudaStreamWaitEvent(to, fork_ev_[ev], 0), "fork wait");
        };
        if (pt && (tail & kTailTransform)) {
            link(s, bt, 6);
            launch_tri_transform(T_, B_, d_sc_, bt);
        }
        launch_step_counter(K_, 1, s);
        if (!sphere_) launch_update_components(C_, O_, s);
        link(s, br, 7);
        if (rest_branch) rotational(br);
        if (walls) {
            link(br, bw, 0);  // the wall law reads velocities
            contacts(1, bw);
        }
        launch_grid_layout(C_, O_, G_, s);
        if (pt) {
            link(s, bt, 1);
            launch_tri_build(T_, B_, G_, K_.tgover, sm_count_, bt);
        }
        launch_grid_sort(C_, O_, G_, sm_count_, s);
        if (O_.ugx) launch_universal_gravity(O_, s);
        launch_gather_geom(C_, O_, G_, R_, sm_count_, K_.gather_bps, K_, s);
        if (pt) {
            // PT reads the geometry records and the owner state itself
            link(s, bt, 2);
            link(br, bt, 10);
        }
        link(s, br, 9);  // the velocity gather follows the sorted order
        launch_gather_vel<T>(C_, O_, G_, R_, dt_eff, sm_count_, K_.gather_bps, br);
        if (pt) contacts(8 | 16, bt);
        contacts(2, s);
        link(br, s, 11);  // the particle law reads the velocity records
        contacts(4, s);
        if (walls) link(bw, s, 3);
        if (pt) {
            link(bt, s, 4);
            launch_body_reduce<T>(R_, d_sc_, B_, ct, BO_, dt_eff > 0.0, bt);
            download(bt);
        }
        launch_owner_sum<T>(C_, O_, d_sc_, ct, false, nullptr, nullptr, nullptr, nullptr, s);
        if (!pt && nb_ > 0) {
            launch_body_reduce<T>(R_, d_sc_, B_, ct, BO_, dt_eff > 0.0, s);
            download(s);
        }
        // the integrator needs only the owner sum: it overlaps the body
        // reduction and the download the host waits for
        integrate(s);
        if (pt) link(bt, s, 5);
        launch_step_counter(K_, 0, s);
        if (tail & kTailDiag) enqueue_diag_download(s);
    }

    void forces(double dt_eff, bool timed = false, unsigned tail = 0)
    {
        if (precision_ == DEM_PRECISION_MIXED) {
            if (pt_fp32_) enqueue_forces<float, float>(dt_eff, hp32_, hw32_, hb32_, ct32_, timed, tail);
            else enqueue_forces<float, double>(dt_eff, hp32_, hw32_, hb64_, ct32_, timed, tail);
        } else {
            enqueue_forces<double, double>(dt_eff, hp64_, hw64_, hb64_, ct64_, timed, tail);
        }
        check(cudaGetLastError(), "force pipeline launch");
    }

    // The neighbour lists' skin of a scene: a share of the room the cell edge
    // leaves beyond the largest pair (r_i + r_j + skin stays within the edge,
    // so the 27 cells of the build sweep hold every pair to list).
    void set_skin(SceneC& S) const
    {
        const double room = std::max(0.0, S.mesh - 2.0 * S.pad);
        const double skin = nl_skin_frac_ * room * (1.0 - 1e-6);
        S.skin_f = (float)skin;
        S.nl_half2 = 0.25 * skin * skin;
    }
    // The single-pass scans' bounded wait, made to run out (a predecessor
    // tile that never publishes): returns the error word it sets.
    unsigned scan_wait_probe()
    {
        unsigned long long* status = nullptr;
        unsigned* err = nullptr;
        check(cudaMalloc(&status, sizeof(unsigned long long)), "probe");
        check(cudaMalloc(&err, sizeof(unsigned)), "probe");
        unsigned out = 0;
        try {
            check(cudaMemsetAsync(status, 0, sizeof(unsigned long long), stream_), "probe");
            check(cudaMemsetAsync(err, 0, sizeof(unsigned), stream_), "probe");
            launch_scan_wait_probe(status, err, stream_);
            check(cudaGetLastError(), "probe");
            check(cudaMemcpyAsync(&out, err, sizeof out, cudaMemcpyDeviceToHost, stream_), "probe");
            check(cudaStreamSynchronize(stream_), "probe");
        } catch (...) {
            cudaFree(status);
            cudaFree(err);
            throw;
        }
        cudaFree(status);
        cudaFree(err);
        return out;
    }

    // Builds so far and the mean list length (host copies; synchronizes).
    void neighbor_stats(int* builds, double* mean_len, int* max_len = nullptr, int* overflowed = nullptr)
    {
        need_init();
        std::vector<int> cnt(nc_);
        int f[3] = {0, 0, 0};
        check(cudaMemcpyAsync(cnt.data(), K_.nl_cnt, sizeof(int) * nc_, cudaMemcpyDeviceToHost, stream_), "stats");
        check(cudaMemcpyAsync(f, K_.nl_flag, sizeof f, cudaMemcpyDeviceToHost, stream_), "stats");
        check(cudaStreamSynchronize(stream_), "stats");
        if (builds) *builds = f[2];
        if (mean_len) *mean_len = nc_ > 0 ? std::accumulate(cnt.begin(), cnt.end(), 0.0) / nc_ : 0.0;
        if (max_len) *max_len = nc_ > 0 ? *std::max_element(cnt.begin(), cnt.end()) : 0;
        if (overflowed) *overflowed = f[1];
    }
    void nl_request_rebuild()
    {
        check(cudaMemsetAsync(K_.nl_flag, 0x01, sizeof(int), stream_), "neighbour lists");
        check(cudaMemsetAsync(K_.nl_flag + 1, 0, sizeof(int), stream_), "neighbour lists");
    }

    double* pin_body_state() { return static_cast<double*>(pinned_); }
    double* pin_body_result() { return static_cast<double*>(pinned_) + 13 * std::max(nb_, 1); }

    void upload_body_state_async()
    {
        if (nb_ <= 0) return;
        double* p = pin_body_state();
        std::memcpy(p, hbc_.data(), sizeof(double) * 3 * nb_);
        std::memcpy(p + 3 * nb_, hbq_.data(), sizeof(double) * 4 * nb_);
        std::memcpy(p + 7 * nb_, hbv_.data(), sizeof(double) * 3 * nb_);
        std::memcpy(p + 10 * nb_, hbw_.data(), sizeof(double) * 3 * nb_);
        enqueue_body_h2d();
    }
    void enqueue_body_h2d()
    {
        double* p = pin_body_state();
        check(cudaMemcpyAsync(B_.c, p, sizeof(double) * 13 * std::max(nb_, 1), cudaMemcpyHostToDevice, stream_),
              "upload body state");
    }
    void body_forces_from_pinned(double* out)
    {
        const double* r = pin_body_result();
        for (int b = 0; b < nb_; ++b) {
            for (int k = 0; k < 6; ++k) out[6 * b + k] = r[(size_t)b * kBodyFieldCount + k];
            const int s = body_scene_[b];
            if (grav_[s]) for (int a = 0; a < 3; ++a) out[6 * b + a] += gvec_[s][a] * body_mass_[b];
        }
    }

    // computeForces (src/cuda_backend_cuda.cu:383-524)
    int compute_forces(const dem_body_states* bodies, double* body_forces, int diag, bool timed = false)
    {
        need_init();
        cudaStream_t s = stream_;
        if (bodies && nb_ > 0) {
            std::memcpy(hbc_.data(), bodies->center, sizeof(double) * 3 * nb_);
            std::memcpy(hbq_.data(), bodies->quat, sizeof(double) * 4 * nb_);
            std::memcpy(hbv_.data(), bodies->vel, sizeof(double) * 3 * nb_);
            std::memcpy(hbw_.data(), bodies->omega, sizeof(double) * 3 * nb_);
            upload_body_state_async();
        }
        const double dt_eff = step_index_ == 0 ? 0.0 : dt_;
        forces(dt_eff, timed, kTailTransform | (nb_ > 0 && (body_forces || diag) ? kTailD2H : 0u));
        ++step_index_;
        if (diag) return collect_diagnostics(body_forces);
        if (body_forces && nb_ > 0) {
            check(cudaStreamSynchronize(s), "compute forces");
            body_forces_from_pinned(body_forces);
        }
        return DEM_OK;
    }

    // Copy the diagnostics block to its pinned mirror and reset the interval
    // sums (the reference's read-and-reset, src/cuda_backend_cuda.cu:500-508).
    void enqueue_diag_download(cudaStream_t s)
    {
        check(cudaMemcpyAsync(diag_pin_, diag_dev_, diag_bytes_, cudaMemcpyDeviceToHost, s), "download diagnostics");
        if (nb_ > 0)
            check(cudaMemsetAsync(diag_dev_ + kDiagIntervalOff, 0, diag_bytes_ - kDiagIntervalOff, s), "reset intervals");
    }

    // downloaded: the stream already holds the download (a run's last graph).
    int collect_diagnostics(double* body_forces, bool downloaded = false)
    {
        cudaStream_t s = stream_;
        if (!downloaded) enqueue_diag_download(s);
        check(cudaStreamSynchronize(s), "collect diagnostics");
        const int* cnt = reinterpret_cast<const int*>(diag_pin_);
        const unsigned err = *reinterpret_cast<const unsigned*>(diag_pin_ + 64);
        const unsigned long long* rint = reinterpret_cast<const unsigned long long*>(diag_pin_ + kDiagIntervalOff);
        const double* mint = reinterpret_cast<const double*>(rint + (size_t)nb_ * kRegime);
        const unsigned long long native = nb_ > 0 ? *reinterpret_cast<const unsigned long long*>(mint + (size_t)nb_ * kMicro) : 0ull;
        dem_step_stats st{};
        st.particle_contacts = cnt[0];
        st.particle_history_overflows = cnt[1];
        st.body_history_overflows = cnt[2];
        st.particle_history_high_water = cnt[3];
        st.body_history_high_water = cnt[4];
        st.triangle_grid_overflows = cnt[5];
        st.cell_table_overflows = (err & kErrCellCapacity) ? 1 : 0;
        st.body_regime_interval_native_steps = native;
        st.body_candidate_items = cnt[9];
        st.wall_candidates = cnt[10];
        reg_inst_.assign((size_t)kRegime * nb_, 0ull);
        reg_int_.assign(rint, rint + (size_t)kRegime * nb_);
        micro_inst_.assign((size_t)kMicro * nb_, 0.0);
        micro_int_.assign(mint, mint + (size_t)kMicro * nb_);
        if (nb_ > 0) {
            const double* r = pin_body_result();
            double fz = 0.0, md = 0.0;
            int bc = 0;
            for (int b = 0; b < nb_; ++b) {
                const double* x = r + (size_t)b * kBodyFieldCount;
                bc += (int)x[6];
                md = std::max(md, x[7]);
                fz += x[8];
                for (int f = 0; f < kRegime; ++f) reg_inst_[b * kRegime + f] = (unsigned long long)x[9 + f];
                for (int f = 0; f < kMicro; ++f) micro_inst_[b * kMicro + f] = x[16 + f];
            }
            st.body_contacts = bc;
            st.body_max_depth = md;
            st.body_contact_fz = fz;
            if (body_forces) body_forces_from_pinned(body_forces);
        }
        stats_ = st;
        if (err & kErrKeyRange) throw DemError(DEM_ERR_CAPACITY, "component grid coordinate exceeds signed 21-bit hash range");
        if (err & kErrCellCapacity)
            throw DemError(DEM_ERR_CAPACITY, "particle cell box exceeds the dense cell-table capacity; raise dem_options.max_cells");
        if (st.particle_history_overflows)
            throw DemError(DEM_ERR_CAPACITY, "CUDA particle contact-history capacity exceeded; increase kGpuParticleHistorySlots");
        if (st.body_history_overflows)
            throw DemError(DEM_ERR_CAPACITY, "CUDA wall/body contact-history capacity exceeded; increase the configured history slots");
        if (st.triangle_grid_overflows || (err & (kErrTriCapacity | kErrTriRange)))
            throw DemError(DEM_ERR_CAPACITY, "CUDA triangle-grid coordinate/count overflow");
        if (err & kErrScanWait) throw DemError(DEM_ERR_CUDA, "a single-pass scan gave up waiting for a predecessor tile");
        return DEM_OK;
    }

    void leapfrog_init(double h) { need_init(); launch_leapfrog_init(O_, h, stream_); check(cudaGetLastError(), "leapfrog init"); }
    void advance(double dt) { need_init(); launch_advance(O_, dt, stream_); check(cudaGetLastError(), "advance"); }
    void finish(double dt) { need_init(); launch_finish(O_, dt, stream_); check(cudaGetLastError(), "finish"); }

    // ------------------------------------------------------- host MBD step
    // DynEqnBodySet (src/dyneq.cpp:97-130) with Quat2DCM (src/matrixtrans.cpp:36-63).
    void dyn_eqn(const double* F, double* ddu)
    {
        for (int b = 0; b < nb_; ++b) {
            double* d = ddu + 6 * b;
            if (body_state_[b] != 0) { for (int k = 0; k < 6; ++k) d[k] = 0.0; continue; }
            for (int k = 0; k < 3; ++k) d[k] = F[6 * b + k] / body_mass_[b];
            const double* q = &hbq_[4 * b];
            const double qq[10] = {q[0] * q[0], q[1] * q[1], q[2] * q[2], q[3] * q[3], 2.0 * q[0] * q[1], 2.0 * q[0] * q[2],
                                   2.0 * q[0] * q[3], 2.0 * q[1] * q[2], 2.0 * q[1] * q[3], 2.0 * q[2] * q[3]};
            const double M[9] = {qq[0] + qq[1] - qq[2] - qq[3], qq[7] + qq[6], qq[8] - qq[5],
                                 qq[7] - qq[6], qq[0] - qq[1] + qq[2] - qq[3], qq[9] + qq[4],
                                 qq[8] + qq[5], qq[9] - qq[4], qq[0] - qq[1] - qq[2] + qq[3]};
            const double T[3] = {F[6 * b + 3], F[6 * b + 4], F[6 * b + 5]};
            double t[3];
            for (int r = 0; r < 3; ++r) t[r] = M[3 * r] * T[0] + M[3 * r + 1] * T[1] + M[3 * r + 2] * T[2];
            const double* I = &body_inertia_[9 * b];
            const double* w = &hbw_[3 * b];
            d[3] = (t[0] - (I[8] - I[4]) * w[2] * w[1]) / I[0];
            d[4] = (t[1] - (I[0] - I[8]) * w[0] * w[2]) / I[4];
            d[5] = (t[2] - (I[4] - I[0]) * w[1] * w[0]) / I[8];
        }
    }
    static void gama(const double* q, const double* w, double* d)
    {
        d[0] = 0.5 * (-q[1] * w[0] - q[2] * w[1] - q[3] * w[2]);
        d[1] = 0.5 * (q[0] * w[0] + q[2] * w[2] - q[3] * w[1]);
        d[2] = 0.5 * (q[0] * w[1] - q[1] * w[2] + q[3] * w[0]);
        d[3] = 0.5 * (q[0] * w[2] + q[1] * w[1] - q[2] * w[0]);
    }
    static void normalize4(double* q)
    {
        const double len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        if (len > 1e-10) { const double s = 1.0 / len; for (int k = 0; k < 4; ++k) q[k] *= s; }
        else for (int k = 0; k < 4; ++k) q[k] = 0.0;
    }
    // Body half-step update after the loads (src/cuda_simulation_integrator.cpp:348-374, 401-425).
    void body_half_update(bool first, double dt)
    {
        const double half = 0.5 * dt;
        std::vector<double> ddu(6 * nb_);
        dyn_eqn(hbloads_.data(), ddu.data());
        for (int b = 0; b < nb_; ++b) {
            double *hv = &hbhv_[3 * b], *hw = &hbhw_[3 * b], *acc = &hbacc_[3 * b], *dom = &hbdom_[3 * b];
            double *V = &hbv_[3 * b], *W = &hbw_[3 * b];
            for (int a = 0; a < 3; ++a) { acc[a] = ddu[6 * b + a]; dom[a] = ddu[6 * b + 3 + a]; }
            const int st = body_state_[b];
            if (st == 0) {
                for (int a = 0; a < 3; ++a) {
                    if (first) { hv[a] = V[a] + acc[a] * half; hw[a] = W[a] + dom[a] * half; }
                    else { hv[a] += acc[a] * dt; hw[a] += dom[a] * dt; }
                }
            } else if (st == 1) {
                for (int a = 0; a < 3; ++a) {
                    acc[a] = dom[a] = hv[a] = hw[a] = 0.0;
                    if (!first) V[a] = W[a] = 0.0;
                }
            } else {
                for (int a = 0; a < 3; ++a) { hv[a] = V[a]; hw[a] = W[a]; }
            }
            double d[4], q[4];
            gama(&hbq_[4 * b], W, d);
            for (int k = 0; k < 4; ++k) q[k] = hbq_[4 * b + k] + d[k] * half;
            normalize4(q);
            std::memcpy(&hbhq_[4 * b], q, sizeof q);
            gama(q, hw, &hbhdq_[4 * b]);
        }
    }
    void body_position_update(double dt)
    {
        const double half = 0.5 * dt;
        for (int b = 0; b < nb_; ++b) {
            if (body_state_[b] == 1) continue;
            for (int a = 0; a < 3; ++a) hbc_[3 * b + a] += hbhv_[3 * b + a] * dt;
            double q[4];
            for (int k = 0; k < 4; ++k) q[k] = hbq_[4 * b + k] + hbhdq_[4 * b + k] * dt;
            normalize4(q);
            std::memcpy(&hbq_[4 * b], q, sizeof q);
            for (int a = 0; a < 3; ++a) {
                hbv_[3 * b + a] = hbhv_[3 * b + a] + hbacc_[3 * b + a] * half;
                hbw_[3 * b + a] = hbhw_[3 * b + a] + hbdom_[3 * b + a] * half;
            }
        }
    }

    // The pose a force evaluation uses, per body (centre, orientation,
    // velocity, spin), and the reverse mode's record of one step: that pose,
    // the loads and the state after the half update.
    std::vector<double> body_pose() const
    {
        std::vector<double> p(13 * (size_t)nb_);
        for (int b = 0; b < nb_; ++b) {
            double* r = p.data() + 13 * (size_t)b;
            for (int a = 0; a < 3; ++a) { r[a] = hbc_[3 * b + a]; r[7 + a] = hbv_[3 * b + a]; r[10 + a] = hbw_[3 * b + a]; }
            for (int k = 0; k < 4; ++k) r[3 + k] = hbq_[4 * b + k];
        }
        return p;
    }
    void adj_record(const std::vector<double>& pose)
    {
        for (int b = 0; b < nb_; ++b) {
            double r[kBR];
            std::memcpy(r, pose.data() + 13 * (size_t)b, 13 * sizeof(double));
            for (int k = 0; k < 6; ++k) r[kBrF + k] = hbloads_[6 * b + k];
            for (int a = 0; a < 3; ++a) {
                r[kBrHV + a] = hbhv_[3 * b + a]; r[kBrHW + a] = hbhw_[3 * b + a];
                r[kBrAcc + a] = hbacc_[3 * b + a]; r[kBrDom + a] = hbdom_[3 * b + a];
            }
            for (int k = 0; k < 4; ++k) { r[kBrHQ + k] = hbhq_[4 * b + k]; r[kBrHDQ + k] = hbhdq_[4 * b + k]; }
            adj_rec_->insert(adj_rec_->end(), r, r + kBR);
        }
    }

    // IntegrateDem / IntegrateDemMultiBody without output frames.  With
    // `defer` the last step stores the half-step velocities and leaves the
    // half-step quaternion rate pending (hq_pending_): the next run's first
    // advance computes it beside its particle grid, as every step inside a
    // run does, and any other use of the state first completes it (settle).
    void run_steps(int steps, bool defer = false)
    {
        need_init();
        const double dt = dt_;
        if (!started_) {
            dem_body_states bs{hbc_.data(), hbq_.data(), hbv_.data(), hbw_.data()};
            const std::vector<double> pose = adj_rec_ ? body_pose() : std::vector<double>();
            compute_forces(nb_ > 0 ? &bs : nullptr, nb_ > 0 ? hbloads_.data() : nullptr, 1);
            if (!restored_) leapfrog_init(0.5 * dt);
            if (nb_ > 0) body_half_update(true, dt);
            if (adj_rec_ && nb_ > 0) adj_record(pose);
            started_ = true;
        }
        if (steps <= 0) return;
        step_loop(steps, defer);
        collect_diagnostics(nullptr, true);
    }

    // `steps` reference steps after the start: advance, then for every step
    // the captured force evaluation.  All but the last step end with the
    // finish and the first part of the next advance (positions); the next
    // step's graph starts with the second part beside its particle grid.
    // The last step ends with finish alone (its velocity part alone with
    // `defer`).  With bodies the host MBD step runs between graph launches.
    void step_loop(int steps, bool defer = false)
    {
        const bool mbd = nb_ > 0;
        ensure_graphs(mbd);
        for (int s = 0; s < steps; ++s) {
            const bool last = s == steps - 1;
            const int head = s > 0 ? 1 : hq_pending_ ? 3 : 2;
            const int tk = !last ? 0 : defer ? 2 : 1;
            capture(graphs_[graph_index(mbd, head, tk)], mbd, head, tk);
            cudaGraphExec_t g = graphs_[graph_index(mbd, head, tk)];
            std::vector<double> pose;
            if (mbd) {
                body_position_update(dt_);
                double* p = pin_body_state();
                std::memcpy(p, hbc_.data(), sizeof(double) * 3 * nb_);
                std::memcpy(p + 3 * nb_, hbq_.data(), sizeof(double) * 4 * nb_);
                std::memcpy(p + 7 * nb_, hbv_.data(), sizeof(double) * 3 * nb_);
                std::memcpy(p + 10 * nb_, hbw_.data(), sizeof(double) * 3 * nb_);
                if (adj_rec_) pose = body_pose();
            }
            check(cudaGraphLaunch(g, stream_), "cudaGraphLaunch");
            ++step_index_;
            if (head == 3) hq_pending_ = false;
            if (tk == 2) hq_pending_ = true;
            if (mbd) {
                // the loads are on the host once the download's event fires;
                // the particle integrator may still be running
                check(cudaEventSynchronize(body_ready_), "mbd step");
                body_forces_from_pinned(hbloads_.data());
                body_half_update(false, dt_);
                if (adj_rec_) adj_record(pose);
            }
        }
        // the callers synchronize (after their own downloads)
    }

    // head: 1 the previous step's rotational advance, 2 this step's advance,
    // 3 this step's advance with the previous step's quaternion rate;
    // tk: 0 not the last step, 1 the last, 2 the last with the rate deferred
    static int graph_index(bool mbd, int head, int tk) { return (mbd ? 12 : 0) + head * 3 + tk; }

    // Complete a deferred finish: the half-step quaternion rate of the last
    // step run (before anything reads or replaces the particle state).
    void settle()
    {
        if (!hq_pending_) return;
        launch_finish_rot(O_, dt_, stream_);
        check(cudaGetLastError(), "finish");
        hq_pending_ = false;
    }
    Engine& settled()
    {
        settle();
        return *this;
    }

    // Captured force evaluation with dt, optionally with the body upload /
    // load download around it and an advance at its head (head 1: the rest
    // of the previous step's, 2: this step's own, 3: this step's own with the
    // previous step's quaternion rate), followed by finish + the position
    // advance (tk 0), finish (tk 1) or its velocity part (tk 2).
    void capture(cudaGraphExec_t& ex, bool mbd, int head, int tk)
    {
        if (ex) return;
        cudaGraph_t g = nullptr;
        check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
        try {
            if (mbd) enqueue_body_h2d();
            forces(dt_, false, (mbd ? kTailTransform | kTailD2H : 0u) |
                                   (head == 1 ? kHeadRest : head == 2 ? kHeadAdvance : kHeadAdvance | kHeadRest) |
                                   (tk == 0 ? kTailFinishPos : tk == 1 ? kTailFinish | kTailDiag
                                                                       : kTailFinishVel | kTailDiag));
        } catch (...) {
            cudaStreamEndCapture(stream_, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        check(cudaStreamEndCapture(stream_, &g), "end capture");
        check(cudaGraphInstantiate(&ex, g, 0), "graph instantiate");
        cudaGraphDestroy(g);
    }
    // Crossover of the two PT kernels (contact items); captured graphs hold
    // the old value, so they are rebuilt on the next graph launch.
    void set_pt_warp_items(int n)
    {
        need_init();
        check(cudaStreamSynchronize(stream_), "sync");
        K_.pt_warp_items = n;
        for (cudaGraphExec_t& g : graphs_)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    }
    // Blocks per SM of the sweep (0: one thread per component), the gathers
    // and the particle law (0: 16); graphs rebuilt.
    void set_launch(int what, int n)
    {
        need_init();
        check(cudaStreamSynchronize(stream_), "sync");
        if (what == 0) K_.sweep_bps = std::max(0, n);
        else if (what == 1) K_.gather_bps = std::max(1, n);
        else if (what == 2) K_.pp_bps = std::max(0, n);
        else if (what == 3) {
            K_.nl_on = n ? 1 : 0;
            nl_request_rebuild();
        } else if (what == 4) {
            // the skin as a share (per mille) of the room the cells leave
            nl_skin_frac_ = std::min(1000, std::max(0, n)) * 1e-3;
            for (SceneC& S : scenes_h_) set_skin(S);
            check(cudaMemcpy(d_sc_, scenes_h_.data(), sizeof(SceneC) * scenes_h_.size(), cudaMemcpyHostToDevice),
                  "scene constants");
            nl_request_rebuild();
        } else throw DemError(DEM_ERR_INVALID, "unknown launch setting");
        for (cudaGraphExec_t& g : graphs_)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        adj_release_graphs();
    }
    void ensure_graphs(bool mbd)
    {
        for (int head = 1; head <= 2; ++head)
            for (int tk = 0; tk < 2; ++tk)
                capture(graphs_[graph_index(mbd, head, tk)], mbd, head, tk);
    }

    // Time `steps` graph-launched steps (pure DEM) on the device; the state is
    // resident.  Returns milliseconds.
    float time_steps(int steps)
    {
        need_init();
        if (!started_) run_steps(1);
        ensure_graphs(nb_ > 0);
        cudaEvent_t a, b;
        check(cudaEventCreate(&a), "event"); check(cudaEventCreate(&b), "event");
        check(cudaStreamSynchronize(stream_), "sync");
        check(cudaEventRecord(a, stream_), "event");
        step_loop(steps);
        check(cudaEventRecord(b, stream_), "event");
        check(cudaEventSynchronize(b), "event sync");
        float ms = 0;
        check(cudaEventElapsedTime(&ms, a, b), "elapsed");
        cudaEventDestroy(a); cudaEventDestroy(b);
        collect_diagnostics(nullptr, true);  // the last graph downloaded them
        return ms;
    }

    // -------------------------------------------------------------- outputs
    void download_state(double* pos, double* vel, double* omg, double* quat)
    {
        need_init();
        check(cudaStreamSynchronize(stream_), "sync");
        auto get3 = [&](double* out, double* x, double* y, double* z) {
            if (!out) return;
            std::vector<double> a(n_), b(n_), c(n_);
            check(cudaMemcpy(a.data(), x, sizeof(double) * n_, cudaMemcpyDeviceToHost), "download");
            check(cudaMemcpy(b.data(), y, sizeof(double) * n_, cudaMemcpyDeviceToHost), "download");
            check(cudaMemcpy(c.data(), z, sizeof(double) * n_, cudaMemcpyDeviceToHost), "download");
            for (int i = 0; i < n_; ++i) { out[3 * i] = a[i]; out[3 * i + 1] = b[i]; out[3 * i + 2] = c[i]; }
        };
        get3(pos, O_.px, O_.py, O_.pz);
        get3(vel, O_.vx, O_.vy, O_.vz);
        get3(omg, O_.wx, O_.wy, O_.wz);
        if (quat) {
            std::vector<double> a(n_);
            double* src[4] = {O_.qw, O_.qx, O_.qy, O_.qz};
            for (int k = 0; k < 4; ++k) {
                check(cudaMemcpy(a.data(), src[k], sizeof(double) * n_, cudaMemcpyDeviceToHost), "download");
                for (int i = 0; i < n_; ++i) quat[4 * i + k] = a[i];
            }
        }
    }

    void download_owner_fields(double* const* dst, double* const* src, int count, int stride)
    {
        std::vector<double> a(n_);
        for (int k = 0; k < count; ++k) {
            check(cudaMemcpy(a.data(), src[k], sizeof(double) * n_, cudaMemcpyDeviceToHost), "download");
            for (int i = 0; i < n_; ++i) (*dst)[(size_t)stride * i + k] = a[i];
        }
    }

    void download_half(double* vh, double* wh, double* hdq, double* acc, double* aacc)
    {
        need_init();
        check(cudaStreamSynchronize(stream_), "sync");
        if (vh) { double* s[3] = {O_.vhx, O_.vhy, O_.vhz}; download_owner_fields(&vh, s, 3, 3); }
        if (wh) { double* s[3] = {O_.whx, O_.why, O_.whz}; download_owner_fields(&wh, s, 3, 3); }
        if (hdq) { double* s[4] = {O_.hqw, O_.hqx, O_.hqy, O_.hqz}; download_owner_fields(&hdq, s, 4, 4); }
        if (acc) { double* s[3] = {O_.ax, O_.ay, O_.az}; download_owner_fields(&acc, s, 3, 3); }
        if (aacc) { double* s[3] = {O_.awx, O_.awy, O_.awz}; download_owner_fields(&aacc, s, 3, 3); }
    }

    template <typename T> void assemble_forces(Contacts<T>& ct, double* c, double* f, double* w, double* t, double* bp, double* bd)
    {
        const size_t n6 = (size_t)n_ * 6;
        double* buf = arena_tmp_.alloc<double>(n6 * 4, "force output");
        launch_owner_sum<T>(C_, O_, d_sc_, ct, true, buf, buf + n6, buf + 2 * n6, buf + 3 * n6, stream_);
        double* bpd = nullptr;
        double* bdd = nullptr;
        if (nb_ > 0 && (bp || bd)) {
            bpd = arena_tmp_.alloc<double>((size_t)nb_ * n6, "body particle output");
            bdd = arena_tmp_.alloc<double>((size_t)nb_ * n_ * 19, "body detail output");
            launch_body_outputs<T>(C_, O_, B_, d_sc_, ct, bpd, bdd, stream_);
        }
        check(cudaStreamSynchronize(stream_), "assemble forces");
        double* dst[4] = {c, f, w, t};
        for (int k = 0; k < 4; ++k)
            if (dst[k]) check(cudaMemcpy(dst[k], buf + k * n6, n6 * sizeof(double), cudaMemcpyDeviceToHost), "download forces");
        if (bp && bpd) check(cudaMemcpy(bp, bpd, (size_t)nb_ * n6 * sizeof(double), cudaMemcpyDeviceToHost), "download");
        if (bd && bdd) check(cudaMemcpy(bd, bdd, (size_t)nb_ * n_ * 19 * sizeof(double), cudaMemcpyDeviceToHost), "download");
        arena_tmp_.release();
    }
    void download_forces(double* c, double* f, double* w, double* t, double* bp, double* bd)
    {
        need_init();
        if (precision_ == DEM_PRECISION_MIXED) assemble_forces<float>(ct32_, c, f, w, t, bp, bd);
        else assemble_forces<double>(ct64_, c, f, w, t, bp, bd);
    }

    void download_grid(uint64_t* keys, int* ids)
    {
        need_init();
        check(cudaStreamSynchronize(stream_), "sync");
        if (keys) check(cudaMemcpy(keys, G_.sorted_key, sizeof(uint64_t) * nc_, cudaMemcpyDeviceToHost), "download keys");
        if (ids) check(cudaMemcpy(ids, G_.sorted_id, sizeof(int) * nc_, cudaMemcpyDeviceToHost), "download ids");
    }

    template <typename T> void download_hist(const Hist<T>& h, int slots, uint64_t* keys, int* last, double* val)
    {
        const size_t n = (size_t)nc_ * slots;
        // keys and last-seen steps are slot-major on the device, the
        // reference's component-major order here
        if (keys) {
            std::vector<uint64_t> k(n);
            check(cudaMemcpy(k.data(), h.key, n * sizeof(uint64_t), cudaMemcpyDeviceToHost), "download keys");
            for (int c = 0; c < nc_; ++c)
                for (int s = 0; s < slots; ++s) keys[(size_t)c * slots + s] = k[(size_t)s * nc_ + c];
        }
        if (last) {
            std::vector<int> l(n);
            check(cudaMemcpy(l.data(), h.last, n * sizeof(int), cudaMemcpyDeviceToHost), "download last");
            for (int c = 0; c < nc_; ++c)
                for (int s = 0; s < slots; ++s) last[(size_t)c * slots + s] = l[(size_t)s * nc_ + c];
        }
        if (val) {
            std::vector<T> v(n * kHV);
            check(cudaMemcpy(v.data(), h.val, n * kHV * sizeof(T), cudaMemcpyDeviceToHost), "download values");
            for (size_t k = 0; k < n; ++k)
                for (int a = 0; a < 9; ++a) val[9 * k + a] = (double)v[kHV * k + a];
        }
    }
    void download_history(int kind, uint64_t* keys, int* last, double* val)
    {
        need_init();
        check(cudaStreamSynchronize(stream_), "sync");
        const int slots = kind == 0 ? kPSlots : (kind == 1 ? kWSlots : kBSlots);
        if (kind < 0 || kind > 2) throw DemError(DEM_ERR_INVALID, "history kind must be 0, 1 or 2");
        if (kind == 2) {
            if (pt_fp32_) download_hist(hb32_, slots, keys, last, val);
            else download_hist(hb64_, slots, keys, last, val);
        } else if (precision_ == DEM_PRECISION_MIXED) {
            download_hist(kind == 0 ? hp32_ : hw32_, slots, keys, last, val);
        } else {
            download_hist(kind == 0 ? hp64_ : hw64_, slots, keys, last, val);
        }
    }

    template <typename T> void upload_hist(Hist<T>& h, int slots, const uint64_t* keys, const double* val)
    {
        const size_t n = (size_t)nc_ * slots;
        std::vector<uint64_t> kt(n);
        for (int c = 0; c < nc_; ++c)
            for (int s = 0; s < slots; ++s) kt[(size_t)s * nc_ + c] = keys[(size_t)c * slots + s];
        check(cudaMemcpy(h.key, kt.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice), "upload keys");
        std::vector<T> v(n * kHV, T(0));
        for (size_t k = 0; k < n; ++k)
            for (int a = 0; a < 9; ++a) v[kHV * k + a] = (T)val[9 * k + a];
        check(cudaMemcpy(h.val, v.data(), n * kHV * sizeof(T), cudaMemcpyHostToDevice), "upload values");
        check(cudaMemset(h.last, 0xff, n * sizeof(int)), "reset history age");
        std::vector<int> hw(nc_, 0);
        for (int c = 0; c < nc_; ++c)
            for (int s = slots - 1; s >= 0; --s)
                if (keys[(size_t)c * slots + s] != 0) { hw[c] = s + 1; break; }
        check(cudaMemcpy(h.hw, hw.data(), nc_ * sizeof(int), cudaMemcpyHostToDevice), "upload hw");
    }

    // ------------------------------------------------- DMHIST2 checkpoint
    // saveContactHistory (src/cuda_backend_cuda.cu:545-656)
    void save_history(const char* path)
    {
        need_init();
        if (!path) throw DemError(DEM_ERR_INVALID, "NULL path");
        check(cudaStreamSynchronize(stream_), "sync");
        const size_t ps = (size_t)nc_ * kPSlots, ws = (size_t)nc_ * kWSlots, bs = (size_t)nc_ * kBSlots;
        std::vector<uint64_t> pk(ps), wk(ws), bk(bs);
        std::vector<double> pv(ps * 9), wv(ws * 9), bv(bs * 9);
        download_history(0, pk.data(), nullptr, pv.data());
        download_history(1, wk.data(), nullptr, wv.data());
        download_history(2, bk.data(), nullptr, bv.data());
        std::vector<double> st(23 * (size_t)n_);
        {
            std::vector<double> a(n_);
            double* src[23] = {O_.px, O_.py, O_.pz, O_.vx, O_.vy, O_.vz, O_.qw, O_.qx, O_.qy, O_.qz, O_.wx, O_.wy,
                               O_.wz, O_.vhx, O_.vhy, O_.vhz, O_.whx, O_.why, O_.whz, O_.hqw, O_.hqx, O_.hqy, O_.hqz};
            for (int k = 0; k < 23; ++k) {
                check(cudaMemcpy(a.data(), src[k], sizeof(double) * n_, cudaMemcpyDeviceToHost), "checkpoint state");
                for (int i = 0; i < n_; ++i) st[23 * (size_t)i + k] = a[i];
            }
        }
        std::ofstream out(path, std::ios::binary | std::ios::trunc);
        if (!out) throw DemError(DEM_ERR_IO, std::string("cannot create CUDA contact-history checkpoint: ") + path);
        auto wr = [&](const void* p, size_t bytes) { out.write(static_cast<const char*>(p), (std::streamsize)bytes); };
        const char magic[8] = {'D', 'M', 'H', 'I', 'S', 'T', '2', '\0'};
        const uint32_t version = 2, endian = 0x01020304u, owners = (uint32_t)n_, comps = (uint32_t)nc_;
        const uint32_t slots[3] = {kPSlots, kWSlots, kBSlots};
        const uint32_t topo = 2u * sizeof(int32_t) + 4u * sizeof(double), ownrec = sizeof(int32_t) + 23u * sizeof(double);
        wr(magic, 8); wr(&version, 4); wr(&endian, 4); wr(&owners, 4); wr(&comps, 4); wr(slots, 12); wr(&topo, 4); wr(&ownrec, 4);
        for (int c = 0; c < nc_; ++c) {
            const int32_t cid = comp_ids_[c], oid = comp_owner_ids_[c];
            const double geo[4] = {comp_radius_[c], comp_body_[3 * c], comp_body_[3 * c + 1], comp_body_[3 * c + 2]};
            wr(&cid, 4); wr(&oid, 4); wr(geo, 32);
        }
        for (int i = 0; i < n_; ++i) {
            const int32_t oid = owner_ids_[i];
            wr(&oid, 4);
            wr(&st[23 * (size_t)i], 23 * sizeof(double));
        }
        wr(pk.data(), ps * 8); wr(wk.data(), ws * 8); wr(bk.data(), bs * 8);
        wr(pv.data(), ps * 72); wr(wv.data(), ws * 72); wr(bv.data(), bs * 72);
        if (!out) throw DemError(DEM_ERR_IO, std::string("failed to write CUDA contact-history checkpoint: ") + path);
    }

    // loadContactHistory (src/cuda_backend_cuda.cu:658-822)
    void load_history(const char* path)
    {
        need_init();
        if (!path) throw DemError(DEM_ERR_INVALID, "NULL path");
        std::ifstream in(path, std::ios::binary);
        const std::string name(path);
        if (!in) throw DemError(DEM_ERR_IO, "cannot open CUDA contact-history checkpoint: " + name);
        auto rd = [&](void* p, size_t bytes) {
            in.read(static_cast<char*>(p), (std::streamsize)bytes);
            if (!in) throw DemError(DEM_ERR_IO, "truncated CUDA contact-history checkpoint: " + name);
        };
        char magic[8];
        uint32_t version = 0, comps = 0, slots[3] = {0, 0, 0};
        rd(magic, 8); rd(&version, 4);
        const char v1[8] = {'D', 'M', 'H', 'I', 'S', 'T', '1', '\0'}, v2[8] = {'D', 'M', 'H', 'I', 'S', 'T', '2', '\0'};
        restored_ = false;
        std::vector<double> st;
        if (std::memcmp(magic, v1, 8) == 0 && version == 1) {
            rd(&comps, 4); rd(slots, 12);
            bool legacy = sphere_;
            for (int i = 0; i < nc_ && legacy; ++i) legacy = comp_ids_[i] == owner_ids_[i];
            if (!legacy) throw DemError(DEM_ERR_IO, "legacy DMHIST1 checkpoint is forbidden for clump topology: " + name);
        } else if (std::memcmp(magic, v2, 8) == 0 && version == 2) {
            uint32_t endian = 0, owners = 0, topo = 0, ownrec = 0;
            rd(&endian, 4); rd(&owners, 4); rd(&comps, 4); rd(slots, 12); rd(&topo, 4); rd(&ownrec, 4);
            if (endian != 0x01020304u || owners != (uint32_t)n_ || topo != 2u * sizeof(int32_t) + 4u * sizeof(double) ||
                ownrec != sizeof(int32_t) + 23u * sizeof(double))
                throw DemError(DEM_ERR_IO, "incompatible DMHIST2 header: " + name);
            if (comps != (uint32_t)nc_) throw DemError(DEM_ERR_IO, "DMHIST2 component count mismatch: " + name);
            for (uint32_t c = 0; c < comps; ++c) {
                int32_t cid = 0, oid = 0;
                double geo[4];
                rd(&cid, 4); rd(&oid, 4); rd(geo, 32);
                if (cid != comp_ids_[c] || oid != comp_owner_ids_[c] || geo[0] != comp_radius_[c] ||
                    geo[1] != comp_body_[3 * c] || geo[2] != comp_body_[3 * c + 1] || geo[3] != comp_body_[3 * c + 2])
                    throw DemError(DEM_ERR_IO, "DMHIST2 component topology mismatch: " + name);
            }
            st.resize(23 * (size_t)n_);
            for (int i = 0; i < n_; ++i) {
                int32_t oid = 0;
                rd(&oid, 4);
                rd(&st[23 * (size_t)i], 23 * sizeof(double));
                if (oid != owner_ids_[i]) throw DemError(DEM_ERR_IO, "DMHIST2 owner identity mismatch: " + name);
            }
        } else {
            throw DemError(DEM_ERR_IO, "unsupported contact-history checkpoint: " + name);
        }
        if (comps != (uint32_t)nc_ || slots[0] != kPSlots || slots[1] != kWSlots || slots[2] != kBSlots)
            throw DemError(DEM_ERR_IO, "incompatible CUDA contact-history checkpoint: " + name);
        const size_t ps = (size_t)nc_ * kPSlots, ws = (size_t)nc_ * kWSlots, bs = (size_t)nc_ * kBSlots;
        std::vector<uint64_t> pk(ps), wk(ws), bk(bs);
        std::vector<double> pv(ps * 9), wv(ws * 9), bv(bs * 9);
        rd(pk.data(), ps * 8); rd(wk.data(), ws * 8); rd(bk.data(), bs * 8);
        rd(pv.data(), ps * 72); rd(wv.data(), ws * 72); rd(bv.data(), bs * 72);
        char trailing;
        if (in.read(&trailing, 1)) throw DemError(DEM_ERR_IO, "oversized CUDA contact-history checkpoint: " + name);
        check(cudaStreamSynchronize(stream_), "sync");
        if (!st.empty()) {
            std::vector<double> a(n_);
            double* dst[23] = {O_.px, O_.py, O_.pz, O_.vx, O_.vy, O_.vz, O_.qw, O_.qx, O_.qy, O_.qz, O_.wx, O_.wy,
                               O_.wz, O_.vhx, O_.vhy, O_.vhz, O_.whx, O_.why, O_.whz, O_.hqw, O_.hqx, O_.hqy, O_.hqz};
            for (int k = 0; k < 23; ++k) {
                for (int i = 0; i < n_; ++i) a[i] = st[23 * (size_t)i + k];
                check(cudaMemcpy(dst[k], a.data(), sizeof(double) * n_, cudaMemcpyHostToDevice), "restore state");
            }
            restored_ = true;
        }
        if (precision_ == DEM_PRECISION_MIXED) {
            upload_hist(hp32_, kPSlots, pk.data(), pv.data()); upload_hist(hw32_, kWSlots, wk.data(), wv.data());
        } else {
            upload_hist(hp64_, kPSlots, pk.data(), pv.data()); upload_hist(hw64_, kWSlots, wk.data(), wv.data());
        }
        if (pt_fp32_) upload_hist(hb32_, kBSlots, bk.data(), bv.data());
        else upload_hist(hb64_, kBSlots, bk.data(), bv.data());
        check(cudaMemset(K_.step, 0, sizeof(int)), "reset step");
        step_index_ = 0;
        started_ = false;
        if (!sphere_) { launch_update_components(C_, O_, stream_); check(cudaStreamSynchronize(stream_), "sync"); }
    }

    // --------------------------------------------------- reverse mode
    // Gradients of the FP64 step by a hand-written adjoint (dem_adjoint.cu):
    // the forward run keeps checkpoints every K steps; the backward run
    // recomputes each segment from its checkpoint with a per-step tape and
    // sweeps it in reverse.  Spheres, walls and particle contacts in one
    // scene; no rigid bodies.
    // One history kind of a checkpoint, compact: every component's occupied
    // prefix [0, hw) of slots at offset off (an exclusive scan of hw).
    struct AdjHist {
        int* hw = nullptr;                         // [nc]
        int* off = nullptr;                        // [nc + 1]
        uint64_t* key = nullptr;                   // [count]
        int* last = nullptr;                       // [count]
        double* val = nullptr;                     // [count][kHV]
        size_t count = 0;
    };
    struct AdjCkpt {
        double* S = nullptr;                       // owner state [29][n]
        AdjHist h[3];                              // particle, wall, body history
        int* step = nullptr;                       // device step counter
        int step_index = 0;
        bool started = false;
    };
    // One segment's tape: owner states, particle and wall entries with their
    // pre-law histories, per-step counts, the device step index, and the
    // graphs of a taped recompute step and a reverse step (reading Lb[p],
    // writing Lb[1 - p]) on it.  Two of them let the recompute of one
    // segment run while the previous one is swept in reverse.
    struct AdjTape {
        double* S = nullptr;                       // [K + 1][29][n]
        int4 *pp = nullptr, *pw = nullptr;         // [K + 1][cap]
        double *pp_h = nullptr, *pw_h = nullptr;
        int *pp_cnt = nullptr, *pw_cnt = nullptr, *slot = nullptr;
        int4* pb = nullptr;                        // particle-body manifolds [K + 1][cap]
        int* pb_tri = nullptr;
        double* pb_h = nullptr;
        int* pb_cnt = nullptr;
        int* base = nullptr;                       // global step of slot 0 (device)
        cudaGraphExec_t g_fwd = nullptr, g_rev[2] = {nullptr, nullptr};
    };
    struct Adjoint {
        bool ready = false;
        int steps = 0, K = 0, nseg = 0, cap_pp = 0, cap_pw = 0, cap_pb = 0;
        std::vector<AdjCkpt> ck;                   // [0] before the first evaluation, [1 + k] after segment k - 1
        AdjTape tb[2];
        unsigned char* pp_new = nullptr;
        int* overflow = nullptr;
        double *L = nullptr, *Lp = nullptr, *P = nullptr, *T = nullptr, *lh_pp = nullptr, *lh_pw = nullptr;
        double* grads = nullptr;
        double* Lb[2] = {nullptr, nullptr};        // the two adjoint-state buffers L and Lp alternate between
        // rigid bodies: the forward run's records ([steps + 1][nb][kBR],
        // host and device), constants, adjoints, body-history adjoints
        std::vector<double> brec_host;
        double *brec = nullptr, *bcst = nullptr, *Lbody = nullptr, *lh_pb = nullptr;
        // single-pass scan scratch of the compact checkpoints; their bytes
        int* scan_n = nullptr;
        int* scan_tiles = nullptr;
        size_t ckpt_bytes = 0, tape_bytes = 0;
        // the largest counts the forward run saw at its checkpoints: contact
        // sides, particle-wall candidates, body manifolds and items
        int seen_pp = 0, seen_pw = 0, seen_pb = 0;
        // the last backward run's adjoints of the bodies' initial state
        // ([nb][kBL] rows; dynamic bodies only)
        std::vector<double> body_grads;
    };
    void adj_release_graphs()
    {
        for (AdjTape& t : adj_.tb)
            for (cudaGraphExec_t* g : {&t.g_fwd, &t.g_rev[0], &t.g_rev[1]})
                if (*g) { cudaGraphExecDestroy(*g); *g = nullptr; }
    }

    void adj_require() const
    {
        need_init();
        if (precision_ != DEM_PRECISION_FP64)
            throw DemError(DEM_ERR_INVALID, "the adjoint runs on the FP64 form (precision DEM_PRECISION_FP64)");
        if (!sphere_) throw DemError(DEM_ERR_INVALID, "the adjoint covers spheres (one component per owner)");
    }
    AdjCkpt adj_alloc_ckpt()
    {
        AdjCkpt c;
        c.S = adj_arena_.alloc<double>((size_t)kAdjFields * n_, "adjoint checkpoint");
        for (int k = 0; k < (nb_ > 0 ? 3 : 2); ++k) {
            c.h[k].hw = adj_arena_.alloc<int>(nc_, "adjoint checkpoint");
            c.h[k].off = adj_arena_.alloc<int>((size_t)nc_ + 1, "adjoint checkpoint");
        }
        c.step = adj_arena_.alloc<int>(1, "adjoint checkpoint");
        return c;
    }
    Hist<double>& adj_live_hist(int k) { return k == 0 ? hp64_ : k == 1 ? hw64_ : hb64_; }
    static int adj_slots(int k) { return k == 0 ? kPSlots : k == 1 ? kWSlots : kBSlots; }
    // The checkpoint keeps each component's occupied history prefix only
    // (about 0.7 kB per settled sphere against 8.6 kB for every slot).
    void adj_save(AdjCkpt& c)
    {
        Adjoint& A = adj_;
        cudaStream_t s = stream_;
        launch_adj_snapshot(O_, c.S, s);
        const int kinds = nb_ > 0 ? 3 : 2;
        int totals[3] = {0, 0, 0};
        for (int k = 0; k < kinds; ++k) {
            AdjHist& h = c.h[k];
            check(cudaMemcpyAsync(h.hw, adj_live_hist(k).hw, sizeof(int) * nc_, cudaMemcpyDeviceToDevice, s),
                  "adjoint checkpoint");
            launch_scan(h.hw, h.off, A.scan_n, A.scan_tiles, sm_count_, s);
            check(cudaMemcpyAsync(totals + k, h.off + nc_, sizeof(int), cudaMemcpyDeviceToHost, s), "adjoint checkpoint");
        }
        check(cudaStreamSynchronize(s), "adjoint checkpoint");
        for (int k = 0; k < kinds; ++k) {
            AdjHist& h = c.h[k];
            h.count = (size_t)totals[k];
            h.key = adj_arena_.alloc<uint64_t>(h.count, "adjoint checkpoint");
            h.last = adj_arena_.alloc<int>(h.count, "adjoint checkpoint");
            h.val = adj_arena_.alloc<double>(h.count * kHV, "adjoint checkpoint");
            launch_ckpt_pack(adj_live_hist(k), adj_slots(k), nc_, h.off, h.key, h.last, h.val, sm_count_, s);
        }
        check(cudaMemcpyAsync(c.step, K_.step, sizeof(int), cudaMemcpyDeviceToDevice, s), "adjoint checkpoint");
        check(cudaGetLastError(), "adjoint checkpoint");
        A.ckpt_bytes += (size_t)kAdjFields * n_ * 8 + (size_t)kinds * (2 * nc_ + 1) * 4;
        for (int k = 0; k < kinds; ++k) A.ckpt_bytes += c.h[k].count * (12 + 8 * kHV);
        c.step_index = step_index_;
        c.started = started_;
    }
    void adj_restore(AdjCkpt& c)
    {
        cudaStream_t s = stream_;
        launch_adj_restore(O_, c.S, s);
        for (int k = 0; k < (nb_ > 0 ? 3 : 2); ++k) {
            const AdjHist& h = c.h[k];
            launch_ckpt_unpack(adj_live_hist(k), adj_slots(k), nc_, h.hw, h.off, h.key, h.last, h.val, sm_count_, s);
        }
        check(cudaMemcpyAsync(K_.step, c.step, sizeof(int), cudaMemcpyDeviceToDevice, s), "adjoint checkpoint");
        check(cudaGetLastError(), "adjoint restore");
        step_index_ = c.step_index;
        started_ = c.started;
    }

    // dem_adjoint_forward: the first evaluation, the leapfrog start and
    // `steps` steps, keeping a checkpoint every K steps.
    void adjoint_forward(int steps, int K)
    {
        adj_require();
        if (steps < 1 || K < 1) throw DemError(DEM_ERR_INVALID, "adjoint forward: steps and K must be positive");
        if (started_ || step_index_ != 0)
            throw DemError(DEM_ERR_STATE, "adjoint forward starts from a freshly initialized engine");
        adj_release_graphs();
        adj_tape_arena_.release();
        adj_arena_.release();
        adj_ = Adjoint{};
        Adjoint& A = adj_;
        A.steps = steps; A.K = std::min(K, steps); A.nseg = (steps + A.K - 1) / A.K;
        A.scan_n = adj_arena_.upload(&nc_, 1, "adjoint checkpoint", stream_);
        A.scan_tiles = adj_arena_.alloc<int>((size_t)nc_ / 1024 + 64, "adjoint checkpoint");
        for (int k = 0; k < A.nseg + 2; ++k) A.ck.push_back(adj_alloc_ckpt());
        A.pp_new = adj_arena_.alloc<unsigned char>((size_t)nc_ * kPSlots, "adjoint tape");
        A.overflow = adj_arena_.alloc<int>(1, "adjoint tape");
        A.L = adj_arena_.alloc<double>((size_t)kAdjFields * n_, "adjoint state");
        A.Lp = adj_arena_.alloc<double>((size_t)kAdjFields * n_, "adjoint state");
        A.P = adj_arena_.alloc<double>((size_t)kPFields * n_, "adjoint state");
        A.T = adj_arena_.alloc<double>((size_t)kTFields * n_, "adjoint state");
        A.lh_pp = adj_arena_.alloc<double>((size_t)nc_ * kPSlots * kHV, "adjoint history");
        A.lh_pw = adj_arena_.alloc<double>((size_t)nc_ * kWSlots * kHV, "adjoint history");
        A.grads = adj_arena_.alloc<double>((size_t)S_ * 3 * kAdjParams, "adjoint parameters");
        A.Lb[0] = A.L; A.Lb[1] = A.Lp;
        if (nb_ > 0) {
            A.lh_pb = adj_arena_.alloc<double>((size_t)nc_ * kBSlots * kHV, "adjoint history");
            A.Lbody = adj_arena_.alloc<double>((size_t)nb_ * kBL, "adjoint bodies");
            std::vector<double> cst(5 * (size_t)nb_);
            for (int b = 0; b < nb_; ++b) {
                cst[5 * b] = body_mass_[b];
                cst[5 * b + 1] = body_inertia_[9 * b];
                cst[5 * b + 2] = body_inertia_[9 * b + 4];
                cst[5 * b + 3] = body_inertia_[9 * b + 8];
                cst[5 * b + 4] = (double)body_state_[b];
            }
            A.bcst = adj_arena_.upload(cst.data(), cst.size(), "adjoint bodies", stream_);
            A.brec_host.clear();
            A.brec_host.reserve((size_t)(steps + 1) * nb_ * kBR);
            adj_rec_ = &A.brec_host;
        }
        auto seen = [&] {
            A.seen_pp = std::max(A.seen_pp, stats_.particle_contacts);
            A.seen_pw = std::max(A.seen_pw, stats_.wall_candidates);
            A.seen_pb = std::max(A.seen_pb, std::max(stats_.body_contacts, stats_.body_candidate_items));
        };
        try {
            adj_save(A.ck[0]);
            run_steps(0);
            seen();
            adj_save(A.ck[1]);
            for (int k = 0; k < A.nseg; ++k) {
                run_steps(std::min(A.K, A.steps - k * A.K));
                seen();
                adj_save(A.ck[k + 2]);
            }
        } catch (...) {
            adj_rec_ = nullptr;
            throw;
        }
        adj_rec_ = nullptr;
        if (nb_ > 0) A.brec = adj_arena_.upload(A.brec_host.data(), A.brec_host.size(), "adjoint bodies", stream_);
        check(cudaStreamSynchronize(stream_), "adjoint forward");
        A.ready = true;
    }

    // The two segment tapes, with room for cap_pp particle contact sides,
    // cap_pw wall contacts and cap_pb body manifolds per step.  The backward
    // run sizes them from the largest counts its forward run saw and grows a
    // capacity that a recompute overflows.
    void adj_alloc_tapes(int cap_pp, int cap_pw, int cap_pb)
    {
        Adjoint& A = adj_;
        adj_release_graphs();
        adj_tape_arena_.release();
        A.cap_pp = cap_pp;
        A.cap_pw = cap_pw;
        A.cap_pb = nb_ > 0 ? cap_pb : 0;
        const size_t slots = (size_t)A.K + 1;
        DeviceArena& a = adj_tape_arena_;
        for (AdjTape& t : A.tb) {
            t = AdjTape{};
            t.S = a.alloc<double>(slots * kAdjFields * n_, "adjoint tape");
            t.pp = a.alloc<int4>(slots * A.cap_pp, "adjoint tape");
            t.pp_h = a.alloc<double>(slots * A.cap_pp * kHV, "adjoint tape");
            t.pw = a.alloc<int4>(slots * A.cap_pw, "adjoint tape");
            t.pw_h = a.alloc<double>(slots * A.cap_pw * kHV, "adjoint tape");
            t.pp_cnt = a.alloc<int>(slots, "adjoint tape");
            t.pw_cnt = a.alloc<int>(slots, "adjoint tape");
            t.slot = a.alloc<int>(1, "adjoint slot");
            t.base = a.alloc<int>(1, "adjoint slot");
            if (nb_ > 0) {
                t.pb = a.alloc<int4>(slots * A.cap_pb, "adjoint tape");
                t.pb_tri = a.alloc<int>(slots * A.cap_pb * kPbTri, "adjoint tape");
                t.pb_h = a.alloc<double>(slots * A.cap_pb * kHV, "adjoint tape");
                t.pb_cnt = a.alloc<int>(slots, "adjoint tape");
            }
        }
        A.tape_bytes = a.bytes();
    }

    // The tape of step `sl` of buffer 0 (the first evaluation), pointers of
    // its own.
    StepTape adj_tape_step(int sl)
    {
        Adjoint& A = adj_;
        const AdjTape& t = A.tb[0];
        StepTape tp{};
        tp.pp_new = A.pp_new;
        tp.pp = t.pp + (size_t)sl * A.cap_pp; tp.pp_h = t.pp_h + (size_t)sl * A.cap_pp * kHV; tp.pp_cap = A.cap_pp;
        tp.pw = t.pw + (size_t)sl * A.cap_pw; tp.pw_h = t.pw_h + (size_t)sl * A.cap_pw * kHV; tp.pw_cap = A.cap_pw;
        tp.pw_count = t.pw_cnt + sl;
        tp.overflow = A.overflow;
        if (t.pb) {
            tp.pb = t.pb + (size_t)sl * A.cap_pb; tp.pb_tri = t.pb_tri + (size_t)sl * A.cap_pb * kPbTri;
            tp.pb_h = t.pb_h + (size_t)sl * A.cap_pb * kHV; tp.pb_cap = A.cap_pb; tp.pb_count = t.pb_cnt + sl;
        }
        return tp;
    }
    // One recomputed force evaluation with its tape in step `sl` of buffer 0.
    void adj_tape_forces(int sl)
    {
        Adjoint& A = adj_;
        check(cudaMemsetAsync(A.tb[0].pw_cnt + sl, 0, sizeof(int), stream_), "adjoint tape");
        if (A.tb[0].pb_cnt) check(cudaMemsetAsync(A.tb[0].pb_cnt + sl, 0, sizeof(int), stream_), "adjoint tape");
        ct64_.tape = adj_tape_step(sl);
        const double dt_eff = step_index_ == 0 ? 0.0 : dt_;
        forces(dt_eff, false, nb_ > 0 ? kTailTransform : 0u);
        ct64_.tape = StepTape{};
        ++step_index_;
        check(cudaMemcpyAsync(A.tb[0].pp_cnt + sl, K_.ct_total, sizeof(int), cudaMemcpyDeviceToDevice, stream_),
              "adjoint tape");
    }

    // The tape of buffer b with the step as its device index.
    StepTape adj_tape_slotted(int b)
    {
        Adjoint& A = adj_;
        const AdjTape& t = A.tb[b];
        StepTape tp{};
        tp.pp_new = A.pp_new;
        tp.pp = t.pp; tp.pp_h = t.pp_h; tp.pp_cap = A.cap_pp;
        tp.pw = t.pw; tp.pw_h = t.pw_h; tp.pw_cap = A.cap_pw;
        tp.pw_count = t.pw_cnt; tp.pp_count = t.pp_cnt;
        tp.overflow = A.overflow;
        tp.slot = t.slot;
        if (t.pb) {
            tp.pb = t.pb; tp.pb_tri = t.pb_tri; tp.pb_h = t.pb_h; tp.pb_cap = A.cap_pb; tp.pb_count = t.pb_cnt;
        }
        return tp;
    }
    // Per buffer: a recomputed, taped step (snapshot, advance, forces,
    // finish, counts; the slot moves on by one) and the reverse step (the
    // slot back by one, then the step's adjoint) as graphs.
    void adj_capture()
    {
        Adjoint& A = adj_;
        if (A.tb[0].g_fwd) return;
        auto cap = [&](cudaGraphExec_t& ex, auto&& body) {
            cudaGraph_t g = nullptr;
            check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
            try {
                body();
            } catch (...) {
                ct64_.tape = StepTape{};
                cudaStreamEndCapture(stream_, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            check(cudaStreamEndCapture(stream_, &g), "end capture");
            check(cudaGraphInstantiate(&ex, g, 0), "graph instantiate");
            cudaGraphDestroy(g);
        };
        for (int b = 0; b < 2; ++b) {
            AdjTape& t = A.tb[b];
            const StepTape tp = adj_tape_slotted(b);
            cap(t.g_fwd, [&] {
                launch_adj_snapshot(O_, t.S, stream_, t.slot);
                launch_advance(O_, dt_, stream_);
                launch_adj_tape_begin(t.pw_cnt, t.pb_cnt, t.slot, stream_);
                if (nb_ > 0) launch_adj_body_pose(B_, A.brec, t.base, t.slot, stream_);
                ct64_.tape = tp;
                forces(dt_, false, nb_ > 0 ? kTailTransform : 0u);
                ct64_.tape = StepTape{};
                launch_finish(O_, dt_, stream_);
                launch_adj_tape_end(t.pp_cnt, K_.ct_total, t.slot, stream_);
            });
            const AdjBodies ab = adj_bodies(t.base);
            for (int p = 0; p < 2; ++p)
                cap(t.g_rev[p], [&] {
                    launch_adj_slot_add(t.slot, -1, stream_);
                    launch_adj_step(C_, O_, d_sc_, W_, tp, -1, -1, -1, t.S, nullptr, A.Lb[p], A.Lb[1 - p], A.P, A.T,
                                    A.lh_pp, A.lh_pw, A.lh_pb, ab, dt_, dt_, 0, A.grads, S_, sm_count_, stream_,
                                    branch_[0], fork_ev_.data(), adj_fp32_);
                });
        }
    }
    AdjBodies adj_bodies(const int* base) const
    {
        const Adjoint& A = adj_;
        AdjBodies ab{};
        ab.nb = nb_ > 0 ? nb_ : 0;
        ab.rec = A.brec; ab.cst = A.bcst; ab.L = A.Lbody; ab.base = base; ab.local = T_.local; ab.dt = dt_;
        return ab;
    }

    // dem_adjoint_backward: the adjoint of the final positions and velocities
    // in, those of the initial state and of the materials out.
    // A recompute wrote more tape entries than the tapes hold (bits: 1
    // particle contacts, 2 wall contacts, 4 body manifolds).
    struct TapeFull {
        int bits;
    };
    void adjoint_backward(const double* dl_dpos, const double* dl_dvel, const double* dl_dbc, const double* dl_dbv,
                          double* dl_dpos0, double* dl_dvel0, double* dl_domega0, double* dl_dparams)
    {
        adj_require();
        Adjoint& A = adj_;
        if (!A.ready) throw DemError(DEM_ERR_STATE, "adjoint backward needs dem_adjoint_forward first");
        const int worst_pp = 16 * nc_ + 1024, worst_pw = 2 * nc_ + 1024, worst_pb = 2 * nc_ + 1024;
        if (!A.tb[0].S)
            adj_alloc_tapes(std::min(worst_pp, A.seen_pp + A.seen_pp / 2 + nc_ / 8 + 1024),
                            std::min(worst_pw, A.seen_pw + A.seen_pw / 2 + 1024),
                            std::min(worst_pb, 2 * A.seen_pb + 1024));
        for (;;) {
            try {
                adjoint_backward_pass(dl_dpos, dl_dvel, dl_dbc, dl_dbv, dl_dpos0, dl_dvel0, dl_domega0, dl_dparams);
                return;
            } catch (const TapeFull& f) {
                check(cudaDeviceSynchronize(), "adjoint tapes");
                const int pp = (f.bits & 1) ? std::min(worst_pp, 2 * A.cap_pp) : A.cap_pp;
                const int pw = (f.bits & 2) ? std::min(worst_pw, 2 * A.cap_pw) : A.cap_pw;
                const int pb = (f.bits & 4) ? std::min(worst_pb, 2 * A.cap_pb) : A.cap_pb;
                if (pp == A.cap_pp && pw == A.cap_pw && pb == A.cap_pb)
                    throw DemError(DEM_ERR_CAPACITY, "adjoint tape capacity exceeded");
                adj_alloc_tapes(pp, pw, pb);
            }
        }
    }
    void adjoint_backward_pass(const double* dl_dpos, const double* dl_dvel, const double* dl_dbc, const double* dl_dbv,
                               double* dl_dpos0, double* dl_dvel0, double* dl_domega0, double* dl_dparams)
    {
        adj_require();
        Adjoint& A = adj_;
        if (!A.ready) throw DemError(DEM_ERR_STATE, "adjoint backward needs dem_adjoint_forward first");
        cudaStream_t s = stream_;
        const size_t N = (size_t)n_;
        check(cudaMemsetAsync(A.L, 0, sizeof(double) * kAdjFields * N, s), "adjoint");
        check(cudaMemsetAsync(A.lh_pp, 0, sizeof(double) * (size_t)nc_ * kPSlots * kHV, s), "adjoint");
        check(cudaMemsetAsync(A.lh_pw, 0, sizeof(double) * (size_t)nc_ * kWSlots * kHV, s), "adjoint");
        check(cudaMemsetAsync(A.grads, 0, sizeof(double) * S_ * 3 * kAdjParams, s), "adjoint");
        check(cudaMemsetAsync(A.overflow, 0, sizeof(int), s), "adjoint");
        std::vector<double> lbody(nb_ > 0 ? (size_t)nb_ * kBL : 0, 0.0);
        if (nb_ > 0) {
            // the loss's adjoint of the final body centres and velocities
            // (the pose of the last evaluation), dynamic bodies only
            for (int b = 0; b < nb_; ++b)
                for (int a = 0; a < 3; ++a) {
                    if (body_state_[b] != 0) continue;
                    if (dl_dbc) lbody[(size_t)b * kBL + kBlC + a] = dl_dbc[3 * b + a];
                    if (dl_dbv) lbody[(size_t)b * kBL + kBlV + a] = dl_dbv[3 * b + a];
                }
            check(cudaMemsetAsync(A.lh_pb, 0, sizeof(double) * (size_t)nc_ * kBSlots * kHV, s), "adjoint");
            check(cudaMemcpyAsync(A.Lbody, lbody.data(), sizeof(double) * lbody.size(), cudaMemcpyHostToDevice, s),
                  "adjoint");
        }
        {
            std::vector<double> h(kAdjFields * N, 0.0);
            for (size_t i = 0; i < N; ++i)
                for (int a = 0; a < 3; ++a) {
                    if (dl_dpos) h[(kAdjX + a) * N + i] = dl_dpos[3 * i + a];
                    if (dl_dvel) h[(kAdjV + a) * N + i] = dl_dvel[3 * i + a];
                }
            check(cudaMemcpyAsync(A.L, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, s), "adjoint");
            check(cudaStreamSynchronize(s), "adjoint");
        }
        std::vector<int> npp(A.K + 1), npw(A.K + 1), npb(A.K + 1, 0);
        auto counts = [&](int k) {
            int of = 0;
            check(cudaMemcpyAsync(npp.data(), A.tb[0].pp_cnt, sizeof(int) * k, cudaMemcpyDeviceToHost, s), "adjoint counts");
            check(cudaMemcpyAsync(npw.data(), A.tb[0].pw_cnt, sizeof(int) * k, cudaMemcpyDeviceToHost, s), "adjoint counts");
            if (A.tb[0].pb_cnt)
                check(cudaMemcpyAsync(npb.data(), A.tb[0].pb_cnt, sizeof(int) * k, cudaMemcpyDeviceToHost, s),
                      "adjoint counts");
            check(cudaMemcpyAsync(&of, A.overflow, sizeof(int), cudaMemcpyDeviceToHost, s), "adjoint counts");
            check(cudaStreamSynchronize(s), "adjoint counts");
            if (of & 8)
                throw DemError(DEM_ERR_CAPACITY, "adjoint tape: a particle-body manifold with more than 12 triangles "
                                                 "with an area share");
            if (of) throw TapeFull{of};
            for (int j = 0; j < k; ++j) {
                npp[j] = std::min(npp[j], A.cap_pp); npw[j] = std::min(npw[j], A.cap_pw); npb[j] = std::min(npb[j], A.cap_pb);
            }
        };
        adj_capture();
        // Segment pipeline: the engine stream recomputes segment k - 1 into
        // one tape while the reverse stream sweeps segment k on the other.
        // The reverse kernels read only the tapes, the adjoint buffers and
        // constant owner data (mass, radius, inertia, status), none of which
        // a recompute writes.
        cudaStream_t rs = branch_[1];  // a high-priority stream (graphs do not use it once captured)
        auto recompute = [&](int seg, int b) {
            AdjTape& t = A.tb[b];
            const int ks = std::min(A.K, A.steps - seg * A.K);
            adj_restore(A.ck[seg + 1]);
            check(cudaMemsetAsync(t.slot, 0, sizeof(int), s), "adjoint slot");
            launch_set_int(t.base, seg * A.K + 1, s);
            for (int sl = 0; sl < ks; ++sl) {
                check(cudaGraphLaunch(t.g_fwd, s), "adjoint recompute");
                ++step_index_;
            }
            launch_adj_snapshot(O_, t.S, s, t.slot);  // the state after the segment, slot ks
            check(cudaEventRecord(adj_ev_[b], s), "adjoint event");
        };
        int par = A.L == A.Lb[0] ? 0 : 1;  // the buffer that holds the current adjoint
        check(cudaEventRecord(adj_ev_[2], s), "adjoint event");
        check(cudaStreamWaitEvent(rs, adj_ev_[2], 0), "adjoint wait");  // the reverse stream after the setup above
        recompute(A.nseg - 1, 0);
        bool rev_used[2] = {false, false};
        for (int seg = A.nseg - 1, b = 0; seg >= 0; --seg, b ^= 1) {
            if (seg > 0) {
                // the other tape was last read by the reverse of segment seg + 1
                if (rev_used[b ^ 1]) check(cudaStreamWaitEvent(s, adj_ev_[3 + (b ^ 1)], 0), "adjoint wait");
                recompute(seg - 1, b ^ 1);
            }
            const int ks = std::min(A.K, A.steps - seg * A.K);
            check(cudaStreamWaitEvent(rs, adj_ev_[b], 0), "adjoint wait");
            for (int sl = ks - 1; sl >= 0; --sl) {
                check(cudaGraphLaunch(A.tb[b].g_rev[par], rs), "adjoint reverse step");
                par ^= 1;
            }
            check(cudaEventRecord(adj_ev_[3 + b], rs), "adjoint event");
            rev_used[b] = true;
        }
        check(cudaEventRecord(adj_ev_[5], rs), "adjoint event");
        check(cudaStreamWaitEvent(s, adj_ev_[5], 0), "adjoint wait");
        A.L = A.Lb[par];
        A.Lp = A.Lb[1 - par];
        // the first evaluation (dt = 0) and the leapfrog start, on tape 0
        adj_restore(A.ck[0]);
        if (nb_ > 0) launch_adj_body_pose(B_, A.brec, nullptr, nullptr, s);
        adj_tape_forces(0);
        launch_leapfrog_init(O_, 0.5 * dt_, s);
        launch_adj_snapshot(O_, A.tb[0].S, s);
        counts(1);
        launch_adj_step(C_, O_, d_sc_, W_, adj_tape_step(0), npp[0], npw[0], npb[0], A.tb[0].S, A.tb[0].S, A.L, A.Lp,
                        A.P, A.T, A.lh_pp, A.lh_pw, A.lh_pb, adj_bodies(nullptr), 0.5 * dt_, 0.0, 1, A.grads, S_,
                        sm_count_, s, nullptr, nullptr, adj_fp32_);
        check(cudaGetLastError(), "adjoint backward");
        std::vector<double> h(kAdjFields * N), g((size_t)S_ * 3 * kAdjParams);
        check(cudaMemcpyAsync(h.data(), A.Lp, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s), "adjoint");
        check(cudaMemcpyAsync(g.data(), A.grads, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, s), "adjoint");
        A.body_grads.assign(nb_ > 0 ? (size_t)nb_ * kBL : 0, 0.0);
        if (nb_ > 0)
            check(cudaMemcpyAsync(A.body_grads.data(), A.Lbody, sizeof(double) * A.body_grads.size(),
                                  cudaMemcpyDeviceToHost, s),
                  "adjoint");
        check(cudaStreamSynchronize(s), "adjoint");
        for (size_t i = 0; i < N; ++i)
            for (int a = 0; a < 3; ++a) {
                if (dl_dpos0) dl_dpos0[3 * i + a] = h[(kAdjX + a) * N + i];
                if (dl_dvel0) dl_dvel0[3 * i + a] = h[(kAdjV + a) * N + i];
                if (dl_domega0) dl_domega0[3 * i + a] = h[(kAdjW + a) * N + i];
            }
        if (dl_dparams)
            for (int sc = 0; sc < S_; ++sc) {
                const MatC* mats[3] = {&scenes_h_[sc].pp, &scenes_h_[sc].pw, &scenes_h_[sc].pt};
                for (int c = 0; c < 3; ++c) {
                    const double* gc = g.data() + ((size_t)sc * 3 + c) * kAdjParams;
                    double* o = dl_dparams + ((size_t)sc * 3 + c) * kAdjParams;
                    // kN, mu, epsN (log epsN = logN), epsS, muT, muR
                    o[0] = gc[0]; o[1] = gc[1];
                    o[2] = gc[2] / std::exp(mats[c]->logN);
                    o[3] = gc[3] / std::exp(mats[c]->logS);
                    o[4] = gc[4]; o[5] = gc[5];
                }
            }
        // leave the engine at the end of the forward run (the host keeps the
        // bodies' end state; their device pose is put back)
        adj_restore(A.ck[A.nseg + 1]);
        if (nb_ > 0) upload_body_state_async();
        check(cudaStreamSynchronize(s), "adjoint backward");
    }

    // -------------------------------------------------------------- misc
    void need_init() const
    {
        if (!initialized_) throw DemError(DEM_ERR_STATE, "CUDA DEM solver is not initialized");
    }

    int n_ = 0, nc_ = 0, nw_ = 0, nb_ = 0, nt_ = 0, S_ = 0, nbs_ = 0;
    bool sphere_ = true, initialized_ = false, started_ = false, restored_ = false;
    bool hq_pending_ = false;  // the last run deferred its quaternion rate (run_steps)
    bool keep_bp_ = false, keep_bd_ = false;
    int precision_ = 0, block_ = 128, sm_count_ = 0;
    bool pt_fp32_ = false;
    double cell_factor_ = 2.5, mesh_ = 0.0, max_radius_ = 0.0, dt_ = 0.0;
    double nl_skin_frac_ = 0.5;
    int step_index_ = 0;
    size_t free_before_ = 0;
    cudaStream_t stream_ = nullptr;
    // Branches of a force evaluation: [0] walls, [1] triangle grid + PT +
    // body reduction, [2] the previous step's rotational advance and the
    // velocity gather; forked from and joined back into stream_ by events.
    std::array<cudaStream_t, 3> branch_{};
    std::array<cudaEvent_t, 12> fork_ev_{};
    cudaEvent_t body_ready_ = nullptr;  // recorded after the body-result download
    std::array<cudaEvent_t, 6> adj_ev_{};  // reverse-mode pipeline: tapes recomputed [2], setup, tapes swept [2], end
    std::array<cudaEvent_t, 12> ev_{};
    int n_marks_ = 0;
    DeviceArena arena_, arena_tmp_, adj_arena_, adj_tape_arena_;
    Adjoint adj_;
    // The reverse law of the particle and wall contacts in FP32 (the forward
    // run, the recompute and everything else stay FP64).
    bool adj_fp32_ = false;
    // dem_adjoint_body_gradients: the last backward run's gradients with
    // respect to the bodies' initial centre, orientation, velocity and
    // body-frame spin (zero for prescribed and fixed bodies).
    void adjoint_body_gradients(double* c, double* q, double* v, double* w) const
    {
        const Adjoint& A = adj_;
        if (A.body_grads.size() != (size_t)nb_ * kBL)
            throw DemError(DEM_ERR_STATE, "adjoint body gradients need dem_adjoint_backward first");
        for (int b = 0; b < nb_; ++b) {
            const double* r = A.body_grads.data() + (size_t)b * kBL;
            const bool dyn = body_state_[b] == 0;
            for (int a = 0; a < 3; ++a) {
                if (c) c[3 * b + a] = dyn ? r[kBlC + a] : 0.0;
                if (v) v[3 * b + a] = dyn ? r[kBlV + a] : 0.0;
                if (w) w[3 * b + a] = dyn ? r[kBlW + a] : 0.0;
            }
            for (int a = 0; a < 4; ++a)
                if (q) q[4 * b + a] = dyn ? r[kBlQ + a] : 0.0;
        }
    }
    void set_adjoint_fp32(bool on)
    {
        if (on != adj_fp32_) adj_release_graphs();
        adj_fp32_ = on;
    }
    std::vector<double>* adj_rec_ = nullptr;  // body records of the forward run, while dem_adjoint_forward runs
    std::vector<double> oin_host_;  // owner principal inertia [n][3] (host copy)
    void* pinned_ = nullptr;
    static constexpr size_t kDiagIntervalOff = 72;  // counters [16] int, error word, then the interval sums
    char* diag_dev_ = nullptr;
    char* diag_pin_ = nullptr;
    size_t diag_bytes_ = 0;
    size_t pinned_bytes_ = 0;
    std::array<cudaGraphExec_t, 24> graphs_{};  // by graph_index(bodies, head, tail kind)

    Owners O_{};
    Comps C_{};
    Grid G_{};
    Recs R_{};
    Walls W_{};
    Tris T_{};
    Bodies B_{};
    Counters K_{};
    SceneC* d_sc_ = nullptr;
    std::vector<SceneC> scenes_h_;
    Hist<double> hp64_{}, hw64_{}, hb64_{};
    Hist<float> hp32_{}, hw32_{}, hb32_{};
    Contacts<double> ct64_{};
    Contacts<float> ct32_{};
    BodyOut BO_{};

    std::vector<int> owner_ids_, comp_ids_, comp_owner_ids_, body_state_, body_scene_, grav_;
    std::vector<std::array<double, 3>> gvec_;
    std::vector<double> comp_radius_, comp_body_, body_mass_, body_inertia_;
    std::vector<double> hbc_, hbq_, hbv_, hbw_, hbhv_, hbhw_, hbhq_, hbhdq_, hbacc_, hbdom_, hbloads_;
    dem_step_stats stats_{};
    std::vector<unsigned long long> reg_inst_, reg_int_;
    std::vector<double> micro_inst_, micro_int_;
};

}  // namespace demgb

// ====================================================================== ABI
using demgb::DemError;
using demgb::Engine;

struct dem_engine {
    Engine e;
};

template <typename F> static int guarded(F&& f)
{
    try {
        f();
        demgb::g_last_error.clear();
        return DEM_OK;
    } catch (const DemError& e) {
        demgb::g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        demgb::g_last_error = "host allocation failed";
        return DEM_ERR_INVALID;
    } catch (const std::exception& e) {
        demgb::g_last_error = e.what();
        return DEM_ERR_INVALID;
    }
}

#define NEED(x) do { if (!(x)) throw DemError(DEM_ERR_INVALID, "NULL argument: " #x); } while (0)

extern "C" {

int dem_abi_version(void) { return DEM_GB300_ABI_VERSION; }
const char* dem_last_error(void) { return demgb::g_last_error.c_str(); }

int dem_device_available(void)
{
    int count = 0;
    return cudaGetDeviceCount(&count) == cudaSuccess && count > 0;
}

const char* dem_device_description(void)
{
    static char description[256] = {0};
    if (description[0] == '\0') {
        cudaDeviceProp p{};
        if (cudaGetDeviceProperties(&p, 0) == cudaSuccess)
            std::snprintf(description, sizeof description, "%s, compute capability %d.%d, %.1f GiB", p.name, p.major,
                          p.minor, (double)p.totalGlobalMem / (1024.0 * 1024.0 * 1024.0));
        else
            std::snprintf(description, sizeof description, "unavailable");
    }
    return description;
}

void dem_default_options(dem_options* o)
{
    if (!o) return;
    o->precision = DEM_PRECISION_FP64;
    o->cell_factor = 2.5;
    o->max_cells = 0;
    o->block_size = 0;
    o->pt_fp32 = 0;
}

int dem_create(dem_engine** out)
{
    return guarded([&] { NEED(out); *out = new dem_engine(); });
}

int dem_destroy(dem_engine* e)
{
    return guarded([&] { delete e; });
}

int dem_initialize(dem_engine* e, const dem_scene* scene, const dem_options* options)
{
    return guarded([&] { NEED(e); NEED(scene); e->e.init(scene, 1, options); });
}

int dem_initialize_batch(dem_engine* e, const dem_scene* scenes, int n, const dem_options* options)
{
    return guarded([&] { NEED(e); NEED(scenes); e->e.init(scenes, n, options); });
}

int dem_compute_forces(dem_engine* e, double, const dem_body_states* bodies, double* body_forces, int diag)
{
    return guarded([&] {
        NEED(e);
        if (bodies) { NEED(bodies->center); NEED(bodies->quat); NEED(bodies->vel); NEED(bodies->omega); }
        e->e.settled().compute_forces(bodies, body_forces, diag);
    });
}

int dem_leapfrog_init(dem_engine* e, double h) { return guarded([&] { NEED(e); e->e.settled().leapfrog_init(h); }); }
int dem_leapfrog_advance(dem_engine* e, double dt) { return guarded([&] { NEED(e); e->e.settled().advance(dt); }); }
int dem_leapfrog_finish(dem_engine* e, double dt, double) { return guarded([&] { NEED(e); e->e.settled().finish(dt); }); }
int dem_run_steps(dem_engine* e, int steps) { return guarded([&] { NEED(e); e->e.run_steps(steps, true); }); }

int dem_get_bodies(dem_engine* e, double* c, double* q, double* v, double* w, double* loads)
{
    return guarded([&] {
        NEED(e);
        Engine& x = e->e;
        const size_t nb = (size_t)x.nb_;
        if (c) std::memcpy(c, x.hbc_.data(), 3 * nb * sizeof(double));
        if (q) std::memcpy(q, x.hbq_.data(), 4 * nb * sizeof(double));
        if (v) std::memcpy(v, x.hbv_.data(), 3 * nb * sizeof(double));
        if (w) std::memcpy(w, x.hbw_.data(), 3 * nb * sizeof(double));
        if (loads) std::memcpy(loads, x.hbloads_.data(), 6 * nb * sizeof(double));
    });
}

int dem_save_history(dem_engine* e, const char* path) { return guarded([&] { NEED(e); e->e.settled().save_history(path); }); }
int dem_load_history(dem_engine* e, const char* path) { return guarded([&] { NEED(e); e->e.settled().load_history(path); }); }
int dem_has_restored_leapfrog_state(dem_engine* e, int* r)
{
    return guarded([&] { NEED(e); NEED(r); *r = e->e.restored_ ? 1 : 0; });
}

int dem_download_state(dem_engine* e, double* pos, double* vel, double* omg, double* quat)
{
    return guarded([&] { NEED(e); e->e.settled().download_state(pos, vel, omg, quat); });
}

int dem_download_forces(dem_engine* e, double* c, double* f, double* w, double* t, double* bp, double* bd)
{
    return guarded([&] { NEED(e); e->e.settled().download_forces(c, f, w, t, bp, bd); });
}

int dem_stats(dem_engine* e, dem_step_stats* s) { return guarded([&] { NEED(e); NEED(s); *s = e->e.stats_; }); }

int dem_body_diagnostics(dem_engine* e, uint64_t* ri, uint64_t* rv, double* mi, double* mv)
{
    return guarded([&] {
        NEED(e);
        Engine& x = e->e;
        if (ri && !x.reg_inst_.empty()) std::memcpy(ri, x.reg_inst_.data(), x.reg_inst_.size() * 8);
        if (rv && !x.reg_int_.empty()) std::memcpy(rv, x.reg_int_.data(), x.reg_int_.size() * 8);
        if (mi && !x.micro_inst_.empty()) std::memcpy(mi, x.micro_inst_.data(), x.micro_inst_.size() * 8);
        if (mv && !x.micro_int_.empty()) std::memcpy(mv, x.micro_int_.data(), x.micro_int_.size() * 8);
    });
}

int dem_grid_entry_counts(dem_engine* e, size_t* pe, size_t* te)
{
    return guarded([&] {
        NEED(e);
        Engine& x = e->e;
        if (pe) *pe = (size_t)x.nc_;
        if (te) {
            int tot = 0, total_cells = 0;
            if (x.nt_ > 0) {
                demgb::check(cudaStreamSynchronize(x.stream_), "sync");
                demgb::check(cudaMemcpy(&total_cells, x.G_.total_cells, sizeof(int), cudaMemcpyDeviceToHost), "download");
                demgb::check(cudaMemcpy(&tot, x.T_.tcell_start + total_cells, sizeof(int), cudaMemcpyDeviceToHost), "download");
            }
            *te = (size_t)tot;
        }
    });
}

int dem_device_memory_bytes(dem_engine* e, size_t* bytes)
{
    return guarded([&] {
        NEED(e); NEED(bytes);
        size_t fr = 0, tot = 0;
        demgb::check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
        *bytes = e->e.free_before_ > fr ? e->e.free_before_ - fr : 0;
    });
}

int dem_counts(dem_engine* e, int* n, int* nc, int* nb, int* nt, int* nw)
{
    return guarded([&] {
        NEED(e);
        Engine& x = e->e;
        if (n) *n = x.n_;
        if (nc) *nc = x.nc_;
        if (nb) *nb = x.nb_;
        if (nt) *nt = x.nt_;
        if (nw) *nw = x.nw_;
    });
}

int dem_download_grid(dem_engine* e, uint64_t* k, int* i) { return guarded([&] { NEED(e); e->e.download_grid(k, i); }); }

int dem_download_history(dem_engine* e, int kind, uint64_t* keys, int* last, double* val)
{
    return guarded([&] { NEED(e); e->e.download_history(kind, keys, last, val); });
}

int dem_last_phase_times(dem_engine* e, float* ms, int capacity, int* count)
{
    return guarded([&] {
        NEED(e);
        Engine& x = e->e;
        const int n = std::max(0, x.n_marks_ - 1);
        if (count) *count = n;
        if (ms) {
            demgb::check(cudaStreamSynchronize(x.stream_), "sync");
            for (int k = 0; k < n && k < capacity; ++k)
                demgb::check(cudaEventElapsedTime(ms + k, x.ev_[k], x.ev_[k + 1]), "elapsed");
        }
    });
}

}  // extern "C"

// Engine-internal entry points used by the Python binding for timing and
// parity introspection (not part of the reference-facing ABI).
extern "C" {

int dem_x_compute_forces_timed(dem_engine* e, int diag)
{
    return guarded([&] { NEED(e); e->e.settled().compute_forces(nullptr, nullptr, diag, true); });
}

int dem_x_time_steps(dem_engine* e, int steps, float* ms)
{
    return guarded([&] { NEED(e); NEED(ms); *ms = e->e.settled().time_steps(steps); });
}

int dem_x_download_half(dem_engine* e, double* vh, double* wh, double* hdq, double* acc, double* aacc)
{
    return guarded([&] { NEED(e); e->e.settled().download_half(vh, wh, hdq, acc, aacc); });
}

int dem_x_set_pt_warp_items(dem_engine* e, int n)
{
    return guarded([&] { NEED(e); e->e.set_pt_warp_items(n); });
}

int dem_x_set_launch(dem_engine* e, int what, int blocks_per_sm)
{
    return guarded([&] { NEED(e); e->e.set_launch(what, blocks_per_sm); });
}

int dem_adjoint_forward(dem_engine* e, int steps, int checkpoint_every)
{
    return guarded([&] { NEED(e); e->e.settled().adjoint_forward(steps, checkpoint_every); });
}

int dem_adjoint_backward(dem_engine* e, const double* dl_dpos, const double* dl_dvel, double* dl_dpos0,
                         double* dl_dvel0, double* dl_domega0, double* dl_dparams)
{
    return guarded([&] {
        NEED(e);
        e->e.settled().adjoint_backward(dl_dpos, dl_dvel, nullptr, nullptr, dl_dpos0, dl_dvel0, dl_domega0, dl_dparams);
    });
}

int dem_adjoint_backward_mbd(dem_engine* e, const double* dl_dpos, const double* dl_dvel, const double* dl_dbody_center,
                             const double* dl_dbody_vel, double* dl_dpos0, double* dl_dvel0, double* dl_domega0,
                             double* dl_dparams)
{
    return guarded([&] {
        NEED(e);
        e->e.settled().adjoint_backward(dl_dpos, dl_dvel, dl_dbody_center, dl_dbody_vel, dl_dpos0, dl_dvel0, dl_domega0,
                              dl_dparams);
    });
}

int dem_x_neighbor_stats(dem_engine* e, int* builds, double* mean_length, int* max_length, int* overflowed)
{
    return guarded([&] { NEED(e); e->e.neighbor_stats(builds, mean_length, max_length, overflowed); });
}

int dem_adjoint_body_gradients(dem_engine* e, double* dl_dbody_center0, double* dl_dbody_quat0,
                               double* dl_dbody_vel0, double* dl_dbody_omega0)
{
    return guarded([&] {
        NEED(e);
        e->e.settled().adjoint_body_gradients(dl_dbody_center0, dl_dbody_quat0, dl_dbody_vel0, dl_dbody_omega0);
    });
}

int dem_x_set_adjoint_fp32(dem_engine* e, int on)
{
    return guarded([&] { NEED(e); e->e.settled().set_adjoint_fp32(on != 0); });
}

int dem_x_adjoint_bytes(dem_engine* e, size_t* checkpoints, size_t* tapes)
{
    return guarded([&] {
        NEED(e);
        *checkpoints = e->e.adj_.ckpt_bytes;
        *tapes = e->e.adj_.tape_bytes;
    });
}

int dem_x_scan_wait_probe(dem_engine* e, unsigned* err)
{
    return guarded([&] { NEED(e); NEED(err); *err = e->e.settled().scan_wait_probe(); });
}

int dem_x_synchronize(dem_engine* e)
{
    return guarded([&] { NEED(e); demgb::check(cudaStreamSynchronize(e->e.stream_), "sync"); });
}

}  // extern "C"
