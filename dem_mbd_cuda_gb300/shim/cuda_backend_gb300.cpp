// cuda_backend_gb300.cpp -- the reference's `class CudaDemSolver`
// (include/cuda_backend.h:40-75) implemented over the GB300 engine's C ABI.
//
// Compile this file instead of the reference's src/cuda_backend_cuda.cu and
// src/cuda/*.cu, against the reference's own headers, and link
// libdemgb300.so: the reference's main, simulation, integrator, loaders,
// writers, dyneq and async output sources then run on the GB300 engine
// unchanged.  Status codes become std::runtime_error with the engine's
// message, as the reference's checkCuda does (src/cuda_backend_cuda.cu:28-33).
#include "cuda_backend.h"
#include "force.h"
#include "multibody.h"
#include "particle.h"
#include "simulation.h"

#include "dem_gb300.h"

#include <stdexcept>
#include <string>
#include <vector>

namespace {

void check(int rc)
{
    if (rc != DEM_OK) throw std::runtime_error(dem_last_error());
}

dem_mech to_mech(const MECH& m)
{
    dem_mech r;
    r.epsS = m.epsS; r.mu = m.mu; r.epsN = m.epsN; r.cohesion = m.c;
    r.beta = m.beta; r.muT = m.mu_T; r.muR = m.mu_R; r.kN = m.kN;
    return r;
}

}  // namespace

class CudaDemSolver::Impl {
public:
    ~Impl()
    {
        if (engine) dem_destroy(engine);
    }
    dem_engine* engine = nullptr;
    int n = 0, nb = 0;
    std::vector<double> bc, bq, bv, bw, loads;

    void bodies_from(const BODYSET& b)
    {
        for (int i = 0; i < nb; ++i) {
            for (int a = 0; a < 3; ++a) {
                bc[3 * i + a] = b.body[i].MassCenter[a];
                bv[3 * i + a] = b.body[i].Vel[a];
                bw[3 * i + a] = b.body[i].AngularVel[a];
            }
            for (int a = 0; a < 4; ++a) bq[4 * i + a] = b.body[i].orien[a];
        }
    }
};

CudaDemSolver::CudaDemSolver() : impl_(new Impl)
{
    check(dem_create(&impl_->engine));
}

CudaDemSolver::~CudaDemSolver() = default;

// CudaDemSolver::initialize (src/cuda_backend_cuda.cu:302-381)
void CudaDemSolver::initialize(PARTICLE& p, BODYSET* bodies, const CONTROL& control, const MECH& particleMech,
                               const MECH& bodyMech, const MECH& wallMech, const ODE& ode)
{
    const int n = p.Num;
    std::vector<double> inertia(3 * (size_t)n), pos(3 * (size_t)n), vel(3 * (size_t)n), omg(3 * (size_t)n),
        quat(4 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            inertia[3 * i + a] = p.Inertia[i][a];
            pos[3 * i + a] = p.Pos[i][a];
            vel[3 * i + a] = p.Vel[i][a];
            omg[3 * i + a] = p.AngSpd[i][a];
        }
        for (int a = 0; a < 4; ++a) quat[4 * i + a] = p.Quat[i][a];
    }
    const int nc = p.ComponentNum;
    std::vector<double> coff(3 * (size_t)(nc > 0 ? nc : 0));
    for (int c = 0; c < nc; ++c)
        for (int a = 0; a < 3; ++a) coff[3 * c + a] = p.ComponentPosBody[c][a];
    dem_scene s{};
    s.n_owners = n;
    s.owner_id = p.Number;
    s.owner_status = p.Status;
    s.owner_mass = p.Mass;
    s.owner_radius = p.Radius;
    s.owner_inertia = inertia.data();
    s.owner_pos = pos.data();
    s.owner_vel = vel.data();
    s.owner_omega = omg.data();
    s.owner_quat = quat.data();
    s.n_components = nc;
    s.comp_owner = p.ComponentOwner;
    s.comp_id = p.ComponentId;
    s.comp_radius = p.ComponentRadius;
    s.comp_offset = coff.data();
    std::vector<double> wo, wn;
    if (control.Wall_flag && control.wall.number > 0) {
        for (int w = 0; w < control.wall.number; ++w)
            for (int a = 0; a < 3; ++a) { wo.push_back(control.wall.Orig[w][a]); wn.push_back(control.wall.N[w][a]); }
        s.n_walls = control.wall.number;
        s.wall_origin = wo.data();
        s.wall_normal = wn.data();
    }
    std::vector<double> bm, bin, tri;
    std::vector<int> bst, tb;
    const int nb = bodies ? bodies->Num : 0;
    impl_->nb = nb;
    impl_->bc.assign(3 * nb, 0.0); impl_->bq.assign(4 * nb, 0.0);
    impl_->bv.assign(3 * nb, 0.0); impl_->bw.assign(3 * nb, 0.0);
    impl_->loads.assign(6 * nb, 0.0);
    if (nb > 0) {
        impl_->bodies_from(*bodies);
        for (int b = 0; b < nb; ++b) {
            const BODY& B = bodies->body[b];
            if (B.Size < 0) throw std::runtime_error("body triangle count cannot be negative");
            bm.push_back(B.Mass);
            bst.push_back(B.state);
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) bin.push_back(B.I[r][c]);
            for (int t = 0; t < B.Size; ++t) {
                const STLTetMesh& m = B.Shape[t];
                const vector3d* v[5] = {&m.v1, &m.v2, &m.v3, &m.v4, &m.normal};
                for (const vector3d* x : v)
                    for (int a = 0; a < 3; ++a) tri.push_back((*x)[a]);
                tb.push_back(b);
            }
        }
        s.n_bodies = nb;
        s.body_mass = bm.data();
        s.body_center = impl_->bc.data();
        s.body_quat = impl_->bq.data();
        s.body_vel = impl_->bv.data();
        s.body_omega = impl_->bw.data();
        s.body_inertia = bin.data();
        s.body_state = bst.data();
        s.n_triangles = (int)tb.size();
        s.tri_body = tb.data();
        s.tri_local = tri.data();
    }
    s.pp = to_mech(particleMech);
    s.pt = to_mech(bodyMech);
    s.pw = to_mech(wallMech);
    s.dt = ode.StepSize;
    for (int a = 0; a < 3; ++a) s.gravity[a] = control.g[a];
    s.gravity_enabled = control.Grav_flag ? 1 : 0;
    s.universal_gravity_enabled = control.Universal_gravitation_flag ? 1 : 0;
    s.keep_body_particle = control.OutputParticleForce ? 1 : 0;
    s.keep_body_detail = control.OutputBodyForce ? 1 : 0;
    check(dem_initialize(impl_->engine, &s, nullptr));
    impl_->n = n;
}

// CudaDemSolver::computeForces (src/cuda_backend_cuda.cu:383-524)
void CudaDemSolver::computeForces(double time, BODYSET* bodies, double** bodyForces, bool collectDiagnostics)
{
    Impl& m = *impl_;
    dem_body_states st{m.bc.data(), m.bq.data(), m.bv.data(), m.bw.data()};
    const bool have = bodies && bodies->Num > 0 && m.nb > 0;
    if (have) m.bodies_from(*bodies);
    double* out = (bodyForces && m.nb > 0) ? m.loads.data() : nullptr;
    check(dem_compute_forces(m.engine, time, have ? &st : nullptr, out, collectDiagnostics ? 1 : 0));
    if (out)
        for (int b = 0; b < m.nb; ++b)
            for (int k = 0; k < 6; ++k) bodyForces[b][k] = m.loads[6 * b + k];
}

void CudaDemSolver::initializeParticleHalfStep(double halfDt) { check(dem_leapfrog_init(impl_->engine, halfDt)); }

double CudaDemSolver::advanceParticles(double fullDt)
{
    check(dem_leapfrog_advance(impl_->engine, fullDt));
    return 0.0;
}

void CudaDemSolver::finishParticleStep(double fullDt, double halfDt)
{
    check(dem_leapfrog_finish(impl_->engine, fullDt, halfDt));
}

void CudaDemSolver::loadContactHistory(const std::string& filename)
{
    check(dem_load_history(impl_->engine, filename.c_str()));
}

void CudaDemSolver::saveContactHistory(const std::string& filename) const
{
    check(dem_save_history(impl_->engine, filename.c_str()));
}

bool CudaDemSolver::hasRestoredParticleLeapfrogState() const
{
    int r = 0;
    check(dem_has_restored_leapfrog_state(impl_->engine, &r));
    return r != 0;
}

// CudaDemSolver::downloadParticleState (src/cuda_backend_cuda.cu:829-846)
void CudaDemSolver::downloadParticleState(PARTICLE& p) const
{
    const int n = impl_->n;
    if (p.Num != n) throw std::runtime_error("particle count changed during CUDA simulation");
    std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), omg(3 * (size_t)n), q(4 * (size_t)n);
    check(dem_download_state(impl_->engine, pos.data(), vel.data(), omg.data(), q.data()));
    for (int i = 0; i < n; ++i) {
        p.Pos[i] = vector3d(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        p.Vel[i] = vector3d(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        p.AngSpd[i] = vector3d(omg[3 * i], omg[3 * i + 1], omg[3 * i + 2]);
        p.Quat[i] = vector4d(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
    }
}

// CudaDemSolver::downloadForceOutput (src/cuda_backend_cuda.cu:848-892)
void CudaDemSolver::downloadForceOutput(FORCE& f, bool particleForces, bool bodyForces) const
{
    const int n = impl_->n, nb = impl_->nb;
    const size_t n6 = (size_t)n * 6;
    std::vector<double> c, fl, w, t, bp, bd;
    if (particleForces) { c.resize(n6); fl.resize(n6); w.resize(n6); t.resize(n6); }
    if (nb > 0 && particleForces) bp.resize((size_t)nb * n6);
    if (nb > 0 && bodyForces) bd.resize((size_t)nb * n * 19);
    check(dem_download_forces(impl_->engine, particleForces ? c.data() : nullptr, particleForces ? fl.data() : nullptr,
                              particleForces ? w.data() : nullptr, particleForces ? t.data() : nullptr,
                              bp.empty() ? nullptr : bp.data(), bd.empty() ? nullptr : bd.data()));
    if (particleForces)
        for (int p = 0; p < n; ++p)
            for (int k = 0; k < 6; ++k) {
                f.Fc[p][k] = c[6 * p + k]; f.Ff[p][k] = fl[6 * p + k]; f.Fw[p][k] = w[6 * p + k];
                f.Fd[p][k] = 0.0; f.FR[p][k] = t[6 * p + k];
            }
    for (int b = 0; b < nb; ++b)
        for (int p = 0; p < n; ++p) {
            if (!bp.empty()) for (int k = 0; k < 6; ++k) f.FI_pt[b][p][k] = bp[((size_t)b * n + p) * 6 + k];
            if (!bd.empty()) for (int k = 0; k < 19; ++k) f.ForceBody[b][p][k] = bd[((size_t)b * n + p) * 19 + k];
        }
    dem_step_stats s{};
    check(dem_stats(impl_->engine, &s));
    f.bodyContactCount = s.body_contacts;
    f.bodyContactMaxDepth = s.body_max_depth;
    f.bodyContactFz = s.body_contact_fz;
}

// CudaDemSolver::stepStats (src/cuda_backend_cuda.cu:894)
CudaStepStats CudaDemSolver::stepStats() const
{
    dem_step_stats s{};
    check(dem_stats(impl_->engine, &s));
    CudaStepStats r;
    r.particleContacts = s.particle_contacts;
    r.bodyContacts = s.body_contacts;
    r.bodyMaxDepth = s.body_max_depth;
    r.bodyContactFz = s.body_contact_fz;
    r.particleHistoryOverflows = s.particle_history_overflows;
    r.bodyHistoryOverflows = s.body_history_overflows;
    r.particleHistoryHighWater = s.particle_history_high_water;
    r.bodyHistoryHighWater = s.body_history_high_water;
    r.triangleGridOverflows = s.triangle_grid_overflows;
    r.bodyRegimeIntervalNativeSteps = s.body_regime_interval_native_steps;
    const int nb = impl_->nb;
    if (nb > 0) {
        std::vector<uint64_t> ri(7 * (size_t)nb), rv(7 * (size_t)nb);
        std::vector<double> mi(22 * (size_t)nb), mv(22 * (size_t)nb);
        check(dem_body_diagnostics(impl_->engine, ri.data(), rv.data(), mi.data(), mv.data()));
        r.bodyRegimeInstant.resize(nb);
        r.bodyRegimeInterval.resize(nb);
        r.bodyMicrostateInstant.resize(nb);
        r.bodyMicrostateInterval.resize(nb);
        for (int b = 0; b < nb; ++b) {
            for (int k = 0; k < 7; ++k) {
                r.bodyRegimeInstant[b][k] = ri[7 * b + k];
                r.bodyRegimeInterval[b][k] = rv[7 * b + k];
            }
            for (int k = 0; k < 22; ++k) {
                r.bodyMicrostateInstant[b][k] = mi[22 * b + k];
                r.bodyMicrostateInterval[b][k] = mv[22 * b + k];
            }
        }
    }
    return r;
}

std::size_t CudaDemSolver::particleGridEntryCount() const
{
    size_t a = 0, b = 0;
    check(dem_grid_entry_counts(impl_->engine, &a, &b));
    return a;
}

std::size_t CudaDemSolver::triangleGridEntryCount() const
{
    size_t a = 0, b = 0;
    check(dem_grid_entry_counts(impl_->engine, &a, &b));
    return b;
}

std::size_t CudaDemSolver::deviceMemoryBytes() const
{
    size_t bytes = 0;
    check(dem_device_memory_bytes(impl_->engine, &bytes));
    return bytes;
}

bool CudaBackendAvailable() { return dem_device_available() != 0; }

const char* CudaDeviceDescription() { return dem_device_description(); }
