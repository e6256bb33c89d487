// ref_cuda_host.cu -- runs the reference's own CUDA engine on a GPU
// (TEST INFRASTRUCTURE ONLY: the checker and the timed FP64 baseline; the
// engine never links or loads it).
//
// The reference's device code is built from its sources where they lie
// (src/cuda/*.cu) into oracle/_ref/ref_engine.cubin by
// oracle/reference_build.py.  Its host glue (src/cuda_backend_cuda.cu and the
// gpu* launch wrappers of src/cuda/*.cu) is C++ that cannot be built for the
// GPU hosts without the reference tree, so this file restates it: the same
// allocations and initial fills, the same kernels in the same order with the
// same launch shapes (256-thread blocks over ceil(n/256) blocks,
// <<<128,256>>> for clearForcesKernel), the same Thrust calls, and the same
// synchronous copies on the legacy default stream.  Kernels are looked up by
// name in the loaded cubin and receive their argument structures byte for
// byte (oracle/ref_cuda_layout.h, checked against the reference's headers).
//
// One difference: a kernel over zero elements is skipped, where the
// reference would fail to launch an empty grid.
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/functional.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <unordered_set>
#include <vector>

#include "../include/dem_gb300.h"
#include "ref_cuda_layout.h"

namespace {

thread_local std::string g_error;

enum Kernel {
    K_UPDATE_COMPONENTS,
    K_COMPONENT_KEYS,
    K_TRANSFORM_TRIANGLES,
    K_COUNT_TRIANGLE_CELLS,
    K_FILL_TRIANGLE_CELLS,
    K_CLEAR_FORCES,
    K_COMPUTE_CONTACTS,
    K_OBSERVE_MICROSTATE,
    K_ACCUMULATE_REGIME,
    K_ACCELERATION,
    K_INIT_LEAPFROG,
    K_ADVANCE_POSITION,
    K_ADVANCE_HALF_VELOCITY,
    K_COUNT
};

const char* const kKernelShortNames[K_COUNT] = {
    "particle.updateComponentsKernel",   "grid.computeComponentKeysKernel",
    "body.transformTrianglesKernel",     "contact.countTriangleCellsKernel",
    "contact.fillTriangleCellsKernel",   "contact.clearForcesKernel",
    "contact.computeContactsKernel",     "contact.observeBodyMicrostateKernel",
    "contact.accumulateBodyRegimeKernel", "particle.accelerationKernel",
    "particle.initializeLeapfrogKernel", "particle.advancePositionKernel",
    "particle.advanceHalfVelocityKernel"};

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

unsigned blocks256(long long n) { return static_cast<unsigned>((n + 255) / 256); }

struct Solver {
    cudaLibrary_t library = nullptr;
    cudaKernel_t fn[K_COUNT] = {};
    std::vector<void*> allocations;

    RefParticles p{};
    RefComponents c{};
    RefWalls w{};
    RefBodyStates b{};
    RefTriangles t{};
    RefGrid grid{};
    RefTriangleGrid tg{};
    RefHistory h{};
    RefForces f{};
    RefMech pm{}, bm{}, wm{};
    int step_index = 0;
    double mesh_size = 0.0, max_radius = 0.0;
    unsigned long long regime_interval_steps = 0;
    dem_step_stats stats{};
    std::vector<unsigned long long> regime_instant, regime_interval;
    std::vector<double> micro_instant, micro_interval;

    int n = 0, nc = 0, nb = 0, nt = 0, nw = 0;
    bool gravity = false;
    double g[3] = {0, 0, 0};
    double dt = 0.0;

    // host MBD state (src/cuda_simulation_integrator.cpp:288-446, src/dyneq.cpp:97-130)
    std::vector<double> bmass, binertia, bc, bq, bv, bw, bhalf_v, bhalf_w, bhalf_q, bhalf_dq, bacc, bdomg, bloads;
    std::vector<int> bstate;
    bool started = false;

    template <typename T>
    T* alloc(size_t count)
    {
        if (count == 0) return nullptr;
        void* ptr = nullptr;
        check(cudaMalloc(&ptr, sizeof(T) * count), "cudaMalloc");
        allocations.push_back(ptr);
        check(cudaMemset(ptr, 0, sizeof(T) * count), "cudaMemset");
        return static_cast<T*>(ptr);
    }

    template <typename... A>
    void launch(Kernel k, unsigned grid_blocks, A... args)
    {
        if (grid_blocks == 0) return;
        void* params[] = {static_cast<void*>(&args)...};
        check(cudaLaunchKernel(reinterpret_cast<const void*>(fn[k]), dim3(grid_blocks), dim3(256), params, 0, 0),
              kKernelShortNames[k]);
    }

    ~Solver()
    {
        for (void* ptr : allocations) cudaFree(ptr);
        if (library) cudaLibraryUnload(library);
    }
};

template <typename T>
void upload(T* dst, const T* src, size_t count, const char* what)
{
    if (count == 0) return;
    check(cudaMemcpy(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice), what);
}

template <typename T>
void download(T* dst, const T* src, size_t count, const char* what)
{
    if (count == 0) return;
    check(cudaMemcpy(dst, src, sizeof(T) * count, cudaMemcpyDeviceToHost), what);
}

void upload_column(double* dst, const double* src, int count, int stride, int col, const char* what)
{
    std::vector<double> v(static_cast<size_t>(count));
    for (int i = 0; i < count; ++i) v[i] = src[static_cast<size_t>(i) * stride + col];
    upload(dst, v.data(), v.size(), what);
}

void download_column(double* dst, const double* src, int count, int stride, int col)
{
    std::vector<double> v(static_cast<size_t>(count));
    download(v.data(), src, v.size(), "download column");
    for (int i = 0; i < count; ++i) dst[static_cast<size_t>(i) * stride + col] = v[i];
}

// uploadBodyStates (src/cuda_backend_cuda.cu:205-227): 13 synchronous copies.
void upload_body_states(Solver& s, const double* c, const double* q, const double* v, const double* w)
{
    upload_column(s.b.cx, c, s.nb, 3, 0, "upload body cx");
    upload_column(s.b.cy, c, s.nb, 3, 1, "upload body cy");
    upload_column(s.b.cz, c, s.nb, 3, 2, "upload body cz");
    upload_column(s.b.qw, q, s.nb, 4, 0, "upload body qw");
    upload_column(s.b.qx, q, s.nb, 4, 1, "upload body qx");
    upload_column(s.b.qy, q, s.nb, 4, 2, "upload body qy");
    upload_column(s.b.qz, q, s.nb, 4, 3, "upload body qz");
    upload_column(s.b.vx, v, s.nb, 3, 0, "upload body vx");
    upload_column(s.b.vy, v, s.nb, 3, 1, "upload body vy");
    upload_column(s.b.vz, v, s.nb, 3, 2, "upload body vz");
    upload_column(s.b.wx, w, s.nb, 3, 0, "upload body wx");
    upload_column(s.b.wy, w, s.nb, 3, 1, "upload body wy");
    upload_column(s.b.wz, w, s.nb, 3, 2, "upload body wz");
}

void transform_triangles(Solver& s) { s.launch(K_TRANSFORM_TRIANGLES, blocks256(s.t.n), s.t, s.b); }

// gpuBuildComponentGrid (src/cuda/cuda_grid_backend.cu:121-145).
void build_component_grid(Solver& s)
{
    s.grid.invMeshSize = 1.0 / s.mesh_size;
    thrust::device_ptr<uint64_t> keys(s.grid.sortedCellKey);
    thrust::device_ptr<int> ids(s.grid.sortedEntityId);
    thrust::sequence(ids, ids + s.grid.n);
    check(cudaMemset(s.grid.overflowCount, 0, sizeof(int)), "clear component grid overflow counter");
    s.launch(K_COMPONENT_KEYS, blocks256(s.grid.n), s.grid, s.c);
    int overflow = 0;
    download(&overflow, s.grid.overflowCount, 1, "copy component grid overflow counter");
    if (overflow != 0) throw std::runtime_error("component grid coordinate exceeds signed 21-bit hash range");
    thrust::sort_by_key(keys, keys + s.grid.n, ids);
}

// gpuBuildTriangleGrid (src/cuda/cuda_contact_backend.cu:1567-1610).
void build_triangle_grid(Solver& s)
{
    RefTriangleGrid& g = s.tg;
    if (g.triangleCount <= 0) {
        g.entryCount = 0;
        return;
    }
    g.invMeshSize = 1.0 / s.mesh_size;
    g.padding = s.max_radius;
    check(cudaMemset(g.overflowCount, 0, sizeof(int)), "clear triangle grid overflow");
    s.launch(K_COUNT_TRIANGLE_CELLS, blocks256(g.triangleCount), g, s.t);
    thrust::device_ptr<int> counts(g.counts), offsets(g.offsets);
    const unsigned long long total =
        thrust::reduce(counts, counts + g.triangleCount, 0ull, thrust::plus<unsigned long long>());
    int overflow = 0;
    download(&overflow, g.overflowCount, 1, "copy triangle grid overflow");
    if (overflow != 0 || total > static_cast<unsigned long long>(INT_MAX))
        throw std::runtime_error("triangle grid entry count exceeds the supported 32-bit index range");
    g.entryCount = static_cast<int>(total);
    if (g.entryCount > g.capacity) {
        // The reference frees and reallocates here; the old arrays stay in
        // the allocation list until destruction.
        g.sortedCellKey = s.alloc<uint64_t>(g.entryCount);
        g.sortedTriangleId = s.alloc<int>(g.entryCount);
        g.capacity = g.entryCount;
    }
    thrust::exclusive_scan(counts, counts + g.triangleCount, offsets);
    s.launch(K_FILL_TRIANGLE_CELLS, blocks256(g.triangleCount), g, s.t);
    thrust::device_ptr<uint64_t> keys(g.sortedCellKey);
    thrust::device_ptr<int> tid(g.sortedTriangleId);
    thrust::sort_by_key(keys, keys + g.entryCount, tid);
}

void to_ref_mech(const dem_mech& m, double dt, RefMech& r)
{
    r = RefMech{};
    r.epsS = m.epsS;
    r.mu = m.mu;
    r.epsN = m.epsN;
    r.cohesion = m.cohesion;
    r.beta = m.beta;
    r.muT = m.muT;
    r.muR = m.muR;
    r.kN = m.kN;
    r.dt = dt;
}

// CudaDemSolver::initialize (src/cuda_backend_cuda.cu:302-381), with
// uploadParticles, uploadComponents, uploadWalls and uploadTriangles
// (:80-255) and the gpuAllocate* functions of src/cuda/*.cu.
void initialize(Solver& s, const dem_scene* sc)
{
    if (!sc || sc->n_owners <= 0) throw std::runtime_error("CUDA DEM solver requires particles");
    {
        std::unordered_set<int> ids;
        for (int i = 0; i < sc->n_owners; ++i)
            if (!ids.insert(sc->owner_id[i]).second)
                throw std::runtime_error("duplicate particle ID " + std::to_string(sc->owner_id[i]) +
                                         "; CUDA contact history requires stable unique particle IDs");
    }
    check(cudaFree(nullptr), "initialize CUDA context");
    const int n = sc->n_owners;
    s.n = n;
    RefParticles& p = s.p;
    p.n = n;
    p.mass = s.alloc<double>(n); p.inertiaX = s.alloc<double>(n); p.inertiaY = s.alloc<double>(n);
    p.inertiaZ = s.alloc<double>(n); p.radius = s.alloc<double>(n); p.id = s.alloc<int>(n);
    p.status = s.alloc<int>(n);
    double** fields[] = {&p.x, &p.y, &p.z, &p.vx, &p.vy, &p.vz, &p.wx, &p.wy, &p.wz, &p.qw, &p.qx, &p.qy,
                         &p.qz, &p.fx, &p.fy, &p.fz, &p.tx, &p.ty, &p.tz, &p.ax, &p.ay, &p.az, &p.awx,
                         &p.awy, &p.awz, &p.vhx, &p.vhy, &p.vhz, &p.whx, &p.why, &p.whz, &p.hdqw, &p.hdqx,
                         &p.hdqy, &p.hdqz, &p.displacement};
    for (double** fp : fields) *fp = s.alloc<double>(n);
    upload(p.mass, sc->owner_mass, n, "upload particle mass");
    upload_column(p.inertiaX, sc->owner_inertia, n, 3, 0, "upload particle inertia x");
    upload_column(p.inertiaY, sc->owner_inertia, n, 3, 1, "upload particle inertia y");
    upload_column(p.inertiaZ, sc->owner_inertia, n, 3, 2, "upload particle inertia z");
    upload(p.radius, sc->owner_radius, n, "upload particle radius");
    upload(p.id, sc->owner_id, n, "upload stable particle id");
    upload(p.status, sc->owner_status, n, "upload particle status");
    double* xyz[] = {p.x, p.y, p.z};
    double* vel[] = {p.vx, p.vy, p.vz};
    double* omg[] = {p.wx, p.wy, p.wz};
    double* quat[] = {p.qw, p.qx, p.qy, p.qz};
    for (int a = 0; a < 3; ++a) {
        upload_column(xyz[a], sc->owner_pos, n, 3, a, "upload position");
        upload_column(vel[a], sc->owner_vel, n, 3, a, "upload velocity");
        upload_column(omg[a], sc->owner_omega, n, 3, a, "upload angular velocity");
    }
    for (int a = 0; a < 4; ++a) upload_column(quat[a], sc->owner_quat, n, 4, a, "upload quaternion");

    // components in (owner, component id) order (uploadComponents, :121-190)
    const int nc = sc->n_components > 0 ? sc->n_components : n;
    s.nc = nc;
    std::vector<int> in_owner(nc), in_id(nc);
    std::vector<double> in_rad(nc), in_off(3 * static_cast<size_t>(nc), 0.0);
    for (int k = 0; k < nc; ++k) {
        if (sc->n_components > 0) {
            in_owner[k] = sc->comp_owner[k];
            in_id[k] = sc->comp_id[k];
            in_rad[k] = sc->comp_radius[k];
            for (int a = 0; a < 3; ++a) in_off[3 * k + a] = sc->comp_offset[3 * k + a];
        } else {
            in_owner[k] = k;
            in_id[k] = sc->owner_id[k];
            in_rad[k] = sc->owner_radius[k];
        }
    }
    std::vector<int> order(nc);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b2) {
        if (in_owner[a] != in_owner[b2]) return in_owner[a] < in_owner[b2];
        return in_id[a] < in_id[b2];
    });
    std::vector<int> cid(nc), cown(nc), ostart(static_cast<size_t>(n) + 1, 0);
    std::vector<double> crad(nc), bx(nc), by(nc), bz(nc);
    double max_r = 0.0;
    for (int k = 0; k < nc; ++k) {
        const int src = order[k];
        if (in_owner[src] < 0 || in_owner[src] >= n || in_id[src] < 0 || !std::isfinite(in_rad[src]) ||
            in_rad[src] <= 0.0)
            throw std::runtime_error("invalid native clump component topology");
        cid[k] = in_id[src];
        cown[k] = in_owner[src];
        crad[k] = in_rad[src];
        bx[k] = in_off[3 * src];
        by[k] = in_off[3 * src + 1];
        bz[k] = in_off[3 * src + 2];
        ++ostart[static_cast<size_t>(cown[k]) + 1];
        max_r = std::max(max_r, crad[k]);
    }
    for (int i = 1; i <= n; ++i) {
        ostart[i] += ostart[i - 1];
        const int count = ostart[i] - ostart[i - 1];
        if (count < 1 || count > 8) throw std::runtime_error("each CUDA owner requires 1 to 8 components");
    }
    RefComponents& c = s.c;
    c.n = nc;
    c.ownerCount = n;
    c.id = s.alloc<int>(nc);
    c.owner = s.alloc<int>(nc);
    c.ownerStart = s.alloc<int>(static_cast<size_t>(n) + 1);
    double** cfields[] = {&c.radius, &c.bodyX, &c.bodyY, &c.bodyZ, &c.offsetX, &c.offsetY, &c.offsetZ, &c.x,
                          &c.y, &c.z, &c.vx, &c.vy, &c.vz, &c.vhx, &c.vhy, &c.vhz};
    for (double** fp : cfields) *fp = s.alloc<double>(nc);
    upload(c.id, cid.data(), nc, "upload component ids");
    upload(c.owner, cown.data(), nc, "upload component owners");
    upload(c.ownerStart, ostart.data(), ostart.size(), "upload component owner starts");
    upload(c.radius, crad.data(), nc, "upload component radii");
    upload(c.bodyX, bx.data(), nc, "upload component body x");
    upload(c.bodyY, by.data(), nc, "upload component body y");
    upload(c.bodyZ, bz.data(), nc, "upload component body z");
    s.launch(K_UPDATE_COMPONENTS, blocks256(nc), s.c, s.p);

    // grid, history (gpuAllocateContactHistory: keys 0, last-seen -1, values 0)
    s.grid.n = nc;
    s.grid.sortedCellKey = s.alloc<uint64_t>(nc);
    s.grid.sortedEntityId = s.alloc<int>(nc);
    s.grid.overflowCount = s.alloc<int>(1);
    RefHistory& h = s.h;
    h.particleCount = nc;
    const size_t ps = static_cast<size_t>(nc) * REF_PARTICLE_SLOTS, ws = static_cast<size_t>(nc) * REF_WALL_SLOTS,
                 bs = static_cast<size_t>(nc) * REF_BODY_SLOTS;
    h.particleKeys = s.alloc<uint64_t>(ps);
    h.wallKeys = s.alloc<uint64_t>(ws);
    h.bodyKeys = s.alloc<uint64_t>(bs);
    h.particleLastSeen = s.alloc<int>(ps);
    h.wallLastSeen = s.alloc<int>(ws);
    h.bodyLastSeen = s.alloc<int>(bs);
    check(cudaMemset(h.particleLastSeen, 0xff, sizeof(int) * ps), "clear particle history age");
    check(cudaMemset(h.wallLastSeen, 0xff, sizeof(int) * ws), "clear wall history age");
    check(cudaMemset(h.bodyLastSeen, 0xff, sizeof(int) * bs), "clear body history age");
    h.particleValues = s.alloc<double>(ps * 9);
    h.wallValues = s.alloc<double>(ws * 9);
    h.bodyValues = s.alloc<double>(bs * 9);

    // forces (gpuAllocateForces, src/cuda/cuda_contact_backend.cu:1415-1525)
    const int nb = sc->n_bodies;
    s.nb = nb;
    RefForces& f = s.f;
    f.particleCount = n;
    f.componentCount = nc;
    f.bodyCount = nb;
    f.contact = s.alloc<double>(6 * static_cast<size_t>(n));
    f.field = s.alloc<double>(6 * static_cast<size_t>(n));
    f.wall = s.alloc<double>(6 * static_cast<size_t>(n));
    f.total = s.alloc<double>(6 * static_cast<size_t>(n));
    if (sc->keep_body_particle) f.bodyParticle = s.alloc<double>(static_cast<size_t>(nb) * n * 6);
    if (sc->keep_body_detail) f.bodyDetail = s.alloc<double>(static_cast<size_t>(nb) * n * 19);
    if (nb > 0) {
        f.bodyRegimeState = s.alloc<int>(static_cast<size_t>(nb) * nc);
        f.bodyMicrostateState = s.alloc<double>(static_cast<size_t>(nb) * nc * REF_MICROSTATE_VALUES);
        f.bodyMicrostateInstant = s.alloc<double>(static_cast<size_t>(nb) * REF_MICROSTATE_VALUES);
        f.bodyMicrostateInterval = s.alloc<double>(static_cast<size_t>(nb) * REF_MICROSTATE_VALUES);
        f.bodyRegimeInstant = s.alloc<unsigned long long>(static_cast<size_t>(nb) * REF_REGIME_COUNTERS);
        f.bodyRegimeInterval = s.alloc<unsigned long long>(static_cast<size_t>(nb) * REF_REGIME_COUNTERS);
    }
    f.bodyResult = s.alloc<double>(6 * static_cast<size_t>(nb));
    f.particleContactCount = s.alloc<int>(1);
    f.bodyContactCount = s.alloc<int>(1);
    f.particleHistoryOverflowCount = s.alloc<int>(1);
    f.bodyHistoryOverflowCount = s.alloc<int>(1);
    f.particleHistoryHighWater = s.alloc<int>(1);
    f.bodyHistoryHighWater = s.alloc<int>(1);
    f.bodyMaxDepth = s.alloc<double>(1);
    f.bodyContactFz = s.alloc<double>(1);

    // walls
    s.nw = sc->n_walls;
    if (s.nw > 0) {
        RefWalls& w = s.w;
        w.n = s.nw;
        double** wf[] = {&w.ox, &w.oy, &w.oz, &w.nx, &w.ny, &w.nz};
        for (double** fp : wf) *fp = s.alloc<double>(s.nw);
        double* o3[] = {w.ox, w.oy, w.oz};
        double* n3[] = {w.nx, w.ny, w.nz};
        for (int a = 0; a < 3; ++a) {
            upload_column(o3[a], sc->wall_origin, s.nw, 3, a, "upload wall origin");
            upload_column(n3[a], sc->wall_normal, s.nw, 3, a, "upload wall normal");
        }
    }

    // bodies and triangles
    if (nb > 0) {
        s.nt = sc->n_triangles;
        RefBodyStates& b = s.b;
        b.n = nb;
        double** bf[] = {&b.cx, &b.cy, &b.cz, &b.qw, &b.qx, &b.qy, &b.qz, &b.vx, &b.vy, &b.vz, &b.wx, &b.wy, &b.wz};
        for (double** fp : bf) *fp = s.alloc<double>(nb);
        RefTriangles& t = s.t;
        t.n = s.nt;
        t.bodyId = s.alloc<int>(s.nt);
        t.triId = s.alloc<int>(s.nt);
        double** tf[] = {&t.lx1, &t.ly1, &t.lz1, &t.lx2, &t.ly2, &t.lz2, &t.lx3, &t.ly3, &t.lz3, &t.lx4,
                         &t.ly4, &t.lz4, &t.lnx, &t.lny, &t.lnz, &t.wx1, &t.wy1, &t.wz1, &t.wx2, &t.wy2,
                         &t.wz2, &t.wx3, &t.wy3, &t.wz3, &t.wx4, &t.wy4, &t.wz4, &t.wnx, &t.wny, &t.wnz,
                         &t.aabbMinX, &t.aabbMinY, &t.aabbMinZ, &t.aabbMaxX, &t.aabbMaxY, &t.aabbMaxZ};
        for (double** fp : tf) *fp = s.alloc<double>(s.nt);
        s.tg.triangleCount = s.nt;
        s.tg.capacity = 0;
        if (s.nt > 0) {
            s.tg.counts = s.alloc<int>(s.nt);
            s.tg.offsets = s.alloc<int>(s.nt);
            s.tg.overflowCount = s.alloc<int>(1);
        }
        upload_body_states(s, sc->body_center, sc->body_quat, sc->body_vel, sc->body_omega);
        // triangle local id = index within its body (uploadTriangles, :229-255)
        std::vector<int> tri_local_id(s.nt);
        std::vector<int> seen(nb, 0);
        for (int k = 0; k < s.nt; ++k) tri_local_id[k] = seen[sc->tri_body[k]]++;
        upload(t.bodyId, sc->tri_body, s.nt, "upload triangle body id");
        upload(t.triId, tri_local_id.data(), s.nt, "upload triangle local id");
        double* loc[] = {t.lx1, t.ly1, t.lz1, t.lx2, t.ly2, t.lz2, t.lx3, t.ly3, t.lz3, t.lx4, t.ly4, t.lz4,
                         t.lnx, t.lny, t.lnz};
        for (int col = 0; col < 15; ++col) upload_column(loc[col], sc->tri_local, s.nt, 15, col, "upload triangle");
        transform_triangles(s);
        s.bmass.assign(sc->body_mass, sc->body_mass + nb);
        s.binertia.assign(sc->body_inertia, sc->body_inertia + 9 * nb);
        s.bstate.assign(sc->body_state, sc->body_state + nb);
        s.bc.assign(sc->body_center, sc->body_center + 3 * nb);
        s.bq.assign(sc->body_quat, sc->body_quat + 4 * nb);
        s.bv.assign(sc->body_vel, sc->body_vel + 3 * nb);
        s.bw.assign(sc->body_omega, sc->body_omega + 3 * nb);
        s.bhalf_v.assign(3 * nb, 0.0);
        s.bhalf_w.assign(3 * nb, 0.0);
        s.bhalf_q.assign(4 * nb, 0.0);
        s.bhalf_dq.assign(4 * nb, 0.0);
        s.bacc.assign(3 * nb, 0.0);
        s.bdomg.assign(3 * nb, 0.0);
        s.bloads.assign(6 * nb, 0.0);
    }
    s.dt = sc->dt;
    to_ref_mech(sc->pp, sc->dt, s.pm);
    to_ref_mech(sc->pt, sc->dt, s.bm);
    to_ref_mech(sc->pw, sc->dt, s.wm);
    s.pm.gx = sc->gravity[0];
    s.pm.gy = sc->gravity[1];
    s.pm.gz = sc->gravity[2];
    s.pm.gravityEnabled = sc->gravity_enabled ? 1 : 0;
    s.pm.universalGravityEnabled = sc->universal_gravity_enabled ? 1 : 0;
    s.gravity = sc->gravity_enabled != 0;
    for (int a = 0; a < 3; ++a) s.g[a] = sc->gravity[a];
    s.mesh_size = 2.5 * max_r;
    s.max_radius = max_r;
    s.regime_instant.assign(static_cast<size_t>(nb) * REF_REGIME_COUNTERS, 0);
    s.regime_interval.assign(static_cast<size_t>(nb) * REF_REGIME_COUNTERS, 0);
    s.micro_instant.assign(static_cast<size_t>(nb) * REF_MICROSTATE_VALUES, 0.0);
    s.micro_interval.assign(static_cast<size_t>(nb) * REF_MICROSTATE_VALUES, 0.0);
}

// CudaDemSolver::computeForces (src/cuda_backend_cuda.cu:383-524).  Returns a
// dem_status; capacity overflows are reported when diagnostics are collected.
int compute_forces(Solver& s, const double* bc, const double* bq, const double* bv, const double* bw,
                   double* body_forces, bool diagnostics)
{
    if (bc && s.nb > 0) {
        upload_body_states(s, bc, bq, bv, bw);
        transform_triangles(s);
    }
    s.launch(K_UPDATE_COMPONENTS, blocks256(s.nc), s.c, s.p);
    build_component_grid(s);
    if (s.t.n > 0) build_triangle_grid(s);
    s.launch(K_CLEAR_FORCES, 128u, s.f);
    const int contact_step = s.step_index++;
    RefMech pm = s.pm, bm = s.bm, wm = s.wm;
    if (contact_step == 0) {
        pm.dt = 0.0;
        bm.dt = 0.0;
        wm.dt = 0.0;
    }
    // gpuComputeContacts (src/cuda/cuda_contact_backend.cu:1618-1647)
    s.launch(K_COMPUTE_CONTACTS, blocks256(s.p.n), s.p, s.c, s.grid, s.w, s.b, s.t, s.tg, s.h, s.f, pm, bm, wm,
             contact_step);
    if (s.f.bodyCount > 0) {
        const long long count = static_cast<long long>(s.f.bodyCount) * s.f.componentCount;
        s.launch(K_OBSERVE_MICROSTATE, blocks256(count), s.p, s.c, s.b, s.t, s.tg, s.h, s.f, bm, contact_step);
        const bool advancing = bm.dt > 0.0;
        s.launch(K_ACCUMULATE_REGIME, blocks256(count), s.f, advancing);
    }
    if (bm.dt > 0.0 && s.b.n > 0) ++s.regime_interval_steps;
    s.launch(K_ACCELERATION, blocks256(s.p.n), s.p);

    int status = DEM_OK;
    if (diagnostics) {
        dem_step_stats st{};
        download(&st.particle_contacts, s.f.particleContactCount, 1, "download particle contact count");
        download(&st.body_contacts, s.f.bodyContactCount, 1, "download body contact count");
        download(&st.body_max_depth, s.f.bodyMaxDepth, 1, "download body max depth");
        download(&st.body_contact_fz, s.f.bodyContactFz, 1, "download body contact Fz");
        if (s.b.n > 0) {
            const size_t count = static_cast<size_t>(s.b.n) * REF_REGIME_COUNTERS;
            download(s.regime_instant.data(), s.f.bodyRegimeInstant, count, "download regime instant");
            download(s.regime_interval.data(), s.f.bodyRegimeInterval, count, "download regime interval");
            st.body_regime_interval_native_steps = s.regime_interval_steps;
            check(cudaMemset(s.f.bodyRegimeInterval, 0, sizeof(unsigned long long) * count),
                  "reset body regime interval counters");
            s.regime_interval_steps = 0;
            const size_t mcount = static_cast<size_t>(s.b.n) * REF_MICROSTATE_VALUES;
            download(s.micro_instant.data(), s.f.bodyMicrostateInstant, mcount, "download microstate instant");
            download(s.micro_interval.data(), s.f.bodyMicrostateInterval, mcount, "download microstate interval");
            check(cudaMemset(s.f.bodyMicrostateInterval, 0, sizeof(double) * mcount),
                  "reset body microstate interval values");
        }
        download(&st.particle_history_overflows, s.f.particleHistoryOverflowCount, 1, "download overflow");
        download(&st.body_history_overflows, s.f.bodyHistoryOverflowCount, 1, "download overflow");
        download(&st.particle_history_high_water, s.f.particleHistoryHighWater, 1, "download high water");
        download(&st.body_history_high_water, s.f.bodyHistoryHighWater, 1, "download high water");
        if (s.tg.overflowCount) download(&st.triangle_grid_overflows, s.tg.overflowCount, 1, "download overflow");
        s.stats = st;
        if (st.particle_history_overflows != 0) {
            g_error = "CUDA particle contact-history capacity exceeded; increase kGpuParticleHistorySlots";
            status = DEM_ERR_CAPACITY;
        } else if (st.body_history_overflows != 0) {
            g_error = "CUDA wall/body contact-history capacity exceeded; increase the configured history slots";
            status = DEM_ERR_CAPACITY;
        } else if (st.triangle_grid_overflows != 0) {
            g_error = "CUDA triangle-grid coordinate/count overflow";
            status = DEM_ERR_CAPACITY;
        }
        if (status != DEM_OK) return status;
    }
    if (body_forces && s.b.n > 0) {
        std::vector<double> result(static_cast<size_t>(s.b.n) * 6);
        download(result.data(), s.f.bodyResult, result.size(), "download body resultant forces");
        for (int body = 0; body < s.b.n; ++body) {
            for (int k = 0; k < 6; ++k) body_forces[6 * body + k] = result[6 * body + k];
            if (s.pm.gravityEnabled) {
                body_forces[6 * body + 0] += s.pm.gx * s.bmass[body];
                body_forces[6 * body + 1] += s.pm.gy * s.bmass[body];
                body_forces[6 * body + 2] += s.pm.gz * s.bmass[body];
            }
        }
    }
    return status;
}

// ------------------------------------------------------------ host MBD step
// gama (src/matrixtrans.cpp:87-96)
void gama(const double* q, const double* w, double* d)
{
    d[0] = 0.5 * (-q[1] * w[0] - q[2] * w[1] - q[3] * w[2]);
    d[1] = 0.5 * (q[0] * w[0] + q[2] * w[2] - q[3] * w[1]);
    d[2] = 0.5 * (q[0] * w[1] - q[1] * w[2] + q[3] * w[0]);
    d[3] = 0.5 * (q[0] * w[2] + q[1] * w[1] - q[2] * w[0]);
}

// vector4d::normalize (include/matrixtrans.h:208-216)
void normalize4(double* q)
{
    const double len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    if (len > 1e-10) {
        const double inv = 1.0 / len;
        for (int k = 0; k < 4; ++k) q[k] *= inv;
    } else {
        for (int k = 0; k < 4; ++k) q[k] = 0.0;
    }
}

// DynEqnBodySet (src/dyneq.cpp:97-130) with Quat2DCM (src/matrixtrans.cpp:36-63)
void dyn_eqn_bodies(const Solver& s, double* ddu)
{
    for (int b = 0; b < s.nb; ++b) {
        double* d = ddu + 6 * b;
        if (s.bstate[b] != 0) {
            for (int k = 0; k < 6; ++k) d[k] = 0.0;
            continue;
        }
        const double* F = s.bloads.data() + 6 * b;
        for (int k = 0; k < 3; ++k) d[k] = F[k] / s.bmass[b];
        const double* q = s.bq.data() + 4 * b;
        const double qq[10] = {q[0] * q[0],       q[1] * q[1],       q[2] * q[2],       q[3] * q[3],
                               2.0 * q[0] * q[1], 2.0 * q[0] * q[2], 2.0 * q[0] * q[3], 2.0 * q[1] * q[2],
                               2.0 * q[1] * q[3], 2.0 * q[2] * q[3]};
        const double M[9] = {qq[0] + qq[1] - qq[2] - qq[3], qq[7] + qq[6], qq[8] - qq[5],
                             qq[7] - qq[6], qq[0] - qq[1] + qq[2] - qq[3], qq[9] + qq[4],
                             qq[8] + qq[5], qq[9] - qq[4], qq[0] - qq[1] - qq[2] + qq[3]};
        double tq[3];
        for (int r = 0; r < 3; ++r) tq[r] = M[3 * r] * F[3] + M[3 * r + 1] * F[4] + M[3 * r + 2] * F[5];
        const double* I = s.binertia.data() + 9 * b;
        const double* w = s.bw.data() + 3 * b;
        d[3] = (tq[0] - (I[8] - I[4]) * w[2] * w[1]) / I[0];
        d[4] = (tq[1] - (I[0] - I[8]) * w[0] * w[2]) / I[4];
        d[5] = (tq[2] - (I[4] - I[0]) * w[1] * w[0]) / I[8];
    }
}

// body half-step update (src/cuda_simulation_integrator.cpp:348-374,402-425)
void body_half_update(Solver& s, bool first, double dt, double half)
{
    std::vector<double> ddu(6 * static_cast<size_t>(s.nb));
    dyn_eqn_bodies(s, ddu.data());
    for (int b = 0; b < s.nb; ++b) {
        double *hv = &s.bhalf_v[3 * b], *hw = &s.bhalf_w[3 * b], *acc = &s.bacc[3 * b], *dom = &s.bdomg[3 * b];
        double *V = &s.bv[3 * b], *W = &s.bw[3 * b];
        for (int a = 0; a < 3; ++a) {
            acc[a] = ddu[6 * b + a];
            dom[a] = ddu[6 * b + 3 + a];
        }
        const int st = s.bstate[b];
        if (st == 0) {
            for (int a = 0; a < 3; ++a) {
                if (first) {
                    hv[a] = V[a] + acc[a] * half;
                    hw[a] = W[a] + dom[a] * half;
                } else {
                    hv[a] += acc[a] * dt;
                    hw[a] += dom[a] * dt;
                }
            }
        } else if (st == 1) {
            for (int a = 0; a < 3; ++a) {
                acc[a] = dom[a] = hv[a] = hw[a] = 0.0;
                if (!first) V[a] = W[a] = 0.0;
            }
        } else {
            for (int a = 0; a < 3; ++a) {
                if (first) acc[a] = dom[a] = 0.0;
                hv[a] = V[a];
                hw[a] = W[a];
            }
        }
        double d[4], q[4];
        gama(&s.bq[4 * b], W, d);
        for (int k = 0; k < 4; ++k) q[k] = s.bq[4 * b + k] + d[k] * half;
        normalize4(q);
        std::memcpy(&s.bhalf_q[4 * b], q, sizeof q);
        gama(q, hw, &s.bhalf_dq[4 * b]);
    }
}

// IntegrateDem / IntegrateDemMultiBody (src/cuda_simulation_integrator.cpp:
// 245-446) without output frames or a prescribed-motion schedule.
int run_steps(Solver& s, int steps)
{
    const double dt = s.dt, half = 0.5 * dt;
    const int nb = s.nb;
    if (!s.started) {
        int rc = compute_forces(s, nb > 0 ? s.bc.data() : nullptr, nb > 0 ? s.bq.data() : nullptr,
                                nb > 0 ? s.bv.data() : nullptr, nb > 0 ? s.bw.data() : nullptr,
                                nb > 0 ? s.bloads.data() : nullptr, true);
        if (rc) return rc;
        s.launch(K_INIT_LEAPFROG, blocks256(s.p.n), s.p, half);
        if (nb > 0) body_half_update(s, true, dt, half);
        s.started = true;
    }
    for (int step = 0; step < steps; ++step) {
        s.launch(K_ADVANCE_POSITION, blocks256(s.p.n), s.p, dt);
        for (int b = 0; b < nb; ++b) {
            if (s.bstate[b] == 1) continue;
            for (int a = 0; a < 3; ++a) s.bc[3 * b + a] += s.bhalf_v[3 * b + a] * dt;
            double q[4];
            for (int k = 0; k < 4; ++k) q[k] = s.bq[4 * b + k] + s.bhalf_dq[4 * b + k] * dt;
            normalize4(q);
            std::memcpy(&s.bq[4 * b], q, sizeof q);
            for (int a = 0; a < 3; ++a) {
                s.bv[3 * b + a] = s.bhalf_v[3 * b + a] + s.bacc[3 * b + a] * half;
                s.bw[3 * b + a] = s.bhalf_w[3 * b + a] + s.bdomg[3 * b + a] * half;
            }
        }
        int rc = compute_forces(s, nb > 0 ? s.bc.data() : nullptr, nb > 0 ? s.bq.data() : nullptr,
                                nb > 0 ? s.bv.data() : nullptr, nb > 0 ? s.bw.data() : nullptr,
                                nb > 0 ? s.bloads.data() : nullptr, step == steps - 1);
        if (rc) return rc;
        s.launch(K_ADVANCE_HALF_VELOCITY, blocks256(s.p.n), s.p, dt);
        if (nb > 0) body_half_update(s, false, dt, half);
    }
    return DEM_OK;
}

template <typename F>
int guarded(F&& body)
{
    try {
        return body();
    } catch (const std::exception& e) {
        g_error = e.what();
        return DEM_ERR_CUDA;
    }
}

}  // namespace

extern "C" {

const char* rfc_error(void) { return g_error.c_str(); }
int rfc_kernel_count(void) { return K_COUNT; }
const char* rfc_kernel_short_name(int k) { return (k >= 0 && k < K_COUNT) ? kKernelShortNames[k] : nullptr; }

// cubin: path of ref_engine.cubin; names: the entry name of each kernel in
// rfc_kernel_short_name order.  Returns NULL on failure (see rfc_error).
void* rfc_create(const char* cubin, const char* const* names, const dem_scene* scene)
{
    Solver* s = new Solver();
    try {
        check(cudaFree(nullptr), "initialize CUDA context");
        check(cudaLibraryLoadFromFile(&s->library, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0),
              "load the reference cubin");
        for (int k = 0; k < K_COUNT; ++k)
            check(cudaLibraryGetKernel(&s->fn[k], s->library, names[k]), kKernelShortNames[k]);
        initialize(*s, scene);
        check(cudaDeviceSynchronize(), "initialize");
        return s;
    } catch (const std::exception& e) {
        g_error = e.what();
        delete s;
        return nullptr;
    }
}

void rfc_destroy(void* h) { delete static_cast<Solver*>(h); }

int rfc_compute_forces(void* h, const double* bc, const double* bq, const double* bv, const double* bw,
                       double* body_forces, int diagnostics)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        const bool have = bc != nullptr;
        if (have && s.nb > 0) {
            s.bc.assign(bc, bc + 3 * s.nb);
            s.bq.assign(bq, bq + 4 * s.nb);
            s.bv.assign(bv, bv + 3 * s.nb);
            s.bw.assign(bw, bw + 3 * s.nb);
        }
        int rc = compute_forces(s, have ? bc : nullptr, bq, bv, bw, body_forces, diagnostics != 0);
        if (rc == DEM_OK && body_forces && s.nb > 0) s.bloads.assign(body_forces, body_forces + 6 * s.nb);
        check(cudaDeviceSynchronize(), "compute forces");
        return rc;
    });
}

int rfc_leapfrog_init(void* h, double half_dt)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        s.launch(K_INIT_LEAPFROG, blocks256(s.p.n), s.p, half_dt);
        check(cudaDeviceSynchronize(), "initializeLeapfrogKernel");
        return DEM_OK;
    });
}

int rfc_advance(void* h, double dt)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        s.launch(K_ADVANCE_POSITION, blocks256(s.p.n), s.p, dt);
        check(cudaDeviceSynchronize(), "advancePositionKernel");
        return DEM_OK;
    });
}

int rfc_finish(void* h, double dt)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        s.launch(K_ADVANCE_HALF_VELOCITY, blocks256(s.p.n), s.p, dt);
        check(cudaDeviceSynchronize(), "advanceHalfVelocityKernel");
        return DEM_OK;
    });
}

int rfc_run(void* h, int steps)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        int rc = run_steps(s, steps);
        check(cudaDeviceSynchronize(), "run");
        return rc;
    });
}

// Wall-clock seconds of `steps` steps of the reference's step loop (device
// synchronised before and after), the way its own integrator runs them.
int rfc_time_run(void* h, int steps, double* seconds)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        check(cudaDeviceSynchronize(), "sync");
        const auto t0 = std::chrono::steady_clock::now();
        int rc = run_steps(s, steps);
        check(cudaDeviceSynchronize(), "run");
        const auto t1 = std::chrono::steady_clock::now();
        *seconds = std::chrono::duration<double>(t1 - t0).count();
        return rc;
    });
}

void rfc_counts(void* h, int* out)
{
    Solver& s = *static_cast<Solver*>(h);
    out[0] = s.n;
    out[1] = s.nc;
    out[2] = s.nb;
    out[3] = s.nt;
    out[4] = s.nw;
    out[5] = s.tg.entryCount;
}

double rfc_mesh_size(void* h) { return static_cast<Solver*>(h)->mesh_size; }

int rfc_get_state(void* h, double* pos, double* vel, double* omg, double* quat)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        const RefParticles& p = s.p;
        const double* xyz[] = {p.x, p.y, p.z};
        const double* v3[] = {p.vx, p.vy, p.vz};
        const double* w3[] = {p.wx, p.wy, p.wz};
        const double* q4[] = {p.qw, p.qx, p.qy, p.qz};
        for (int a = 0; a < 3; ++a) {
            download_column(pos, xyz[a], s.n, 3, a);
            download_column(vel, v3[a], s.n, 3, a);
            download_column(omg, w3[a], s.n, 3, a);
        }
        for (int a = 0; a < 4; ++a) download_column(quat, q4[a], s.n, 4, a);
        return DEM_OK;
    });
}

int rfc_get_half(void* h, double* vh, double* wh, double* hdq, double* acc, double* aacc)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        const RefParticles& p = s.p;
        const double* a3[][3] = {{p.vhx, p.vhy, p.vhz}, {p.whx, p.why, p.whz}, {p.ax, p.ay, p.az},
                                 {p.awx, p.awy, p.awz}};
        double* out3[] = {vh, wh, acc, aacc};
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) download_column(out3[k], a3[k][a], s.n, 3, a);
        const double* q4[] = {p.hdqw, p.hdqx, p.hdqy, p.hdqz};
        for (int a = 0; a < 4; ++a) download_column(hdq, q4[a], s.n, 4, a);
        return DEM_OK;
    });
}

int rfc_get_forces(void* h, double* contact, double* field, double* wall, double* total, double* body_particle,
                   double* body_detail)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        const size_t n6 = 6 * static_cast<size_t>(s.n);
        download(contact, s.f.contact, n6, "download contact");
        download(field, s.f.field, n6, "download field");
        download(wall, s.f.wall, n6, "download wall");
        download(total, s.f.total, n6, "download total");
        if (body_particle && s.f.bodyParticle)
            download(body_particle, s.f.bodyParticle, static_cast<size_t>(s.nb) * n6, "download body particle");
        if (body_detail && s.f.bodyDetail)
            download(body_detail, s.f.bodyDetail, static_cast<size_t>(s.nb) * s.n * 19, "download body detail");
        return DEM_OK;
    });
}

int rfc_get_grid(void* h, uint64_t* keys, int* ids)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        download(keys, s.grid.sortedCellKey, s.nc, "download sorted keys");
        download(ids, s.grid.sortedEntityId, s.nc, "download sorted ids");
        return DEM_OK;
    });
}

int rfc_get_triangle_grid(void* h, uint64_t* keys, int* ids)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        download(keys, s.tg.sortedCellKey, s.tg.entryCount, "download triangle keys");
        download(ids, s.tg.sortedTriangleId, s.tg.entryCount, "download triangle ids");
        return DEM_OK;
    });
}

int rfc_get_world_triangles(void* h, double* tw, double* aabb)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        const RefTriangles& t = s.t;
        const double* cols[] = {t.wx1, t.wy1, t.wz1, t.wx2, t.wy2, t.wz2, t.wx3, t.wy3,
                                t.wz3, t.wx4, t.wy4, t.wz4, t.wnx, t.wny, t.wnz};
        for (int k = 0; k < 15; ++k) download_column(tw, cols[k], s.nt, 15, k);
        const double* box[] = {t.aabbMinX, t.aabbMinY, t.aabbMinZ, t.aabbMaxX, t.aabbMaxY, t.aabbMaxZ};
        for (int k = 0; k < 6; ++k) download_column(aabb, box[k], s.nt, 6, k);
        return DEM_OK;
    });
}

int rfc_get_components(void* h, double* pos, double* vel, double* vh, double* off)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        const RefComponents& c = s.c;
        const double* cols[][3] = {{c.x, c.y, c.z}, {c.vx, c.vy, c.vz}, {c.vhx, c.vhy, c.vhz},
                                   {c.offsetX, c.offsetY, c.offsetZ}};
        double* out[] = {pos, vel, vh, off};
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) download_column(out[k], cols[k][a], s.nc, 3, a);
        return DEM_OK;
    });
}

int rfc_get_history(void* h, int kind, uint64_t* keys, int* last, double* values)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        const int slots = kind == 0 ? REF_PARTICLE_SLOTS : kind == 1 ? REF_WALL_SLOTS : REF_BODY_SLOTS;
        const uint64_t* k = kind == 0 ? s.h.particleKeys : kind == 1 ? s.h.wallKeys : s.h.bodyKeys;
        const int* l = kind == 0 ? s.h.particleLastSeen : kind == 1 ? s.h.wallLastSeen : s.h.bodyLastSeen;
        const double* v = kind == 0 ? s.h.particleValues : kind == 1 ? s.h.wallValues : s.h.bodyValues;
        const size_t count = static_cast<size_t>(s.nc) * slots;
        download(keys, k, count, "download history keys");
        download(last, l, count, "download history last-seen");
        download(values, v, count * 9, "download history values");
        return DEM_OK;
    });
}

void rfc_get_stats(void* h, dem_step_stats* out) { *out = static_cast<Solver*>(h)->stats; }

void rfc_body_diagnostics(void* h, unsigned long long* ri, unsigned long long* rv, double* mi, double* mv)
{
    Solver& s = *static_cast<Solver*>(h);
    std::copy(s.regime_instant.begin(), s.regime_instant.end(), ri);
    std::copy(s.regime_interval.begin(), s.regime_interval.end(), rv);
    std::copy(s.micro_instant.begin(), s.micro_instant.end(), mi);
    std::copy(s.micro_interval.begin(), s.micro_interval.end(), mv);
}

int rfc_get_regime_state(void* h, int* state)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        download(state, s.f.bodyRegimeState, static_cast<size_t>(s.nb) * s.nc, "download regime state");
        return DEM_OK;
    });
}

int rfc_get_microstate(void* h, double* values)
{
    Solver& s = *static_cast<Solver*>(h);
    return guarded([&] {
        download(values, s.f.bodyMicrostateState, static_cast<size_t>(s.nb) * s.nc * REF_MICROSTATE_VALUES,
                 "download microstate");
        return DEM_OK;
    });
}

void rfc_get_bodies(void* h, double* c, double* q, double* v, double* w, double* loads)
{
    Solver& s = *static_cast<Solver*>(h);
    std::copy(s.bc.begin(), s.bc.end(), c);
    std::copy(s.bq.begin(), s.bq.end(), q);
    std::copy(s.bv.begin(), s.bv.end(), v);
    std::copy(s.bw.begin(), s.bw.end(), w);
    std::copy(s.bloads.begin(), s.bloads.end(), loads);
}

size_t rfc_device_bytes(void* h)
{
    (void)h;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    return total_b - free_b;
}

}  // extern "C"
