// dem_adjoint.cu -- reverse sweep of the FP64 step: kernels.
//
// One step of the engine maps the owner state S_s (29 values per owner,
// layout below) and the contact history to S_{s+1}:
//   advance  x1 = x + vh dt, q1 = N(q + hq dt), v1 = vh + a dt/2, w1 = wh + aw dt/2
//            (advancePositionKernel, src/cuda/cuda_particle_backend.cu:212-237)
//   forces   a1, aw1 from the contact laws at (x1, q1, v1, w1) with the
//            midpoint velocities (vh, wh) (computeContactsKernel and
//            accelerationKernel, src/cuda/cuda_contact_backend.cu:1082-1220,
//            src/cuda/cuda_particle_backend.cu:71-101)
//   finish   vh1 = vh + a1 dt, wh1 = wh + aw1 dt,
//            hq1 = G(N(q1 + dt/2 G(q1, w1)), wh1)  (advanceHalfVelocityKernel,
//            :239-265)
// The reverse sweep runs, per step: the body leapfrog's half-update
// reverse (k_adj_body_a), k_adj_finish (finish^T and the owner part of
// forces^T, Euler's equations with their gyroscopic terms), k_adj_contacts
// (particle and wall contacts, scattering into the owners with FP64
// atomics), k_adj_pt (particle-body manifolds) and the body position
// update's reverse (k_adj_body_c) beside them, then k_adj_advance
// (advance^T).  The history adjoints live in the reference's slot layout, so
// a contact that persists keeps its slot and its adjoint; a slot acquired
// new in the step gets a zero adjoint before it.  Spheres (one component per
// owner) with any principal inertia; dynamic rigid bodies.
#include <algorithm>

#include "dem_adjoint.cuh"
#include "dem_kernels.cuh"

namespace demgb {

namespace {

inline int nblocks(int n, int b) { return (n + b - 1) / b; }

__device__ __forceinline__ D3 ld3(const double* A, int f, int n, int i)
{
    return mk(A[(size_t)f * n + i], A[(size_t)(f + 1) * n + i], A[(size_t)(f + 2) * n + i]);
}
__device__ __forceinline__ void st3(double* A, int f, int n, int i, D3 v)
{
    A[(size_t)f * n + i] = v.x; A[(size_t)(f + 1) * n + i] = v.y; A[(size_t)(f + 2) * n + i] = v.z;
}
__device__ __forceinline__ void ld4(const double* A, int f, int n, int i, double q[4])
{
    for (int k = 0; k < 4; ++k) q[k] = A[(size_t)(f + k) * n + i];
}
__device__ __forceinline__ void st4(double* A, int f, int n, int i, const double q[4])
{
    for (int k = 0; k < 4; ++k) A[(size_t)(f + k) * n + i] = q[k];
}
__device__ __forceinline__ void add3(double* A, int f, int n, int i, D3 v)
{
    atomicAdd(A + (size_t)f * n + i, v.x);
    atomicAdd(A + (size_t)(f + 1) * n + i, v.y);
    atomicAdd(A + (size_t)(f + 2) * n + i, v.z);
}
__device__ __forceinline__ void add4(double* A, int f, int n, int i, const double q[4])
{
    for (int k = 0; k < 4; ++k) atomicAdd(A + (size_t)(f + k) * n + i, q[k]);
}
template <typename R> __device__ __forceinline__ void normq(R q[4])
{
    const R n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (n2 <= R(1.0e-24)) { q[0] = R(1.0); q[1] = q[2] = q[3] = R(0.0); return; }
    R inv;
    if constexpr (std::is_same<R, double>::value) inv = rsqrt(n2);
    else inv = rsqrtf(n2);
    for (int k = 0; k < 4; ++k) q[k] *= inv;
}

// The post-advance state of owner i from S_s (and the midpoint velocities
// the laws use: vh, wh, or the endpoint ones when there is no midpoint).
__device__ void post_advance(const double* S, int n, int i, double dt, bool moves, bool mid, D3& x1, double q1[4], D3& v1,
                             D3& w1, D3& mv, D3& mw)
{
    const D3 x = ld3(S, kAdjX, n, i), vh = ld3(S, kAdjVH, n, i), wh = ld3(S, kAdjWH, n, i);
    double q[4], hq[4];
    ld4(S, kAdjQ, n, i, q);
    ld4(S, kAdjHQ, n, i, hq);
    if (moves) {
        x1 = x + vh * dt;
        for (int k = 0; k < 4; ++k) q1[k] = q[k] + hq[k] * dt;
        normq(q1);
        v1 = vh + ld3(S, kAdjA, n, i) * (0.5 * dt);
        w1 = wh + ld3(S, kAdjAW, n, i) * (0.5 * dt);
    } else {
        x1 = x;
        for (int k = 0; k < 4; ++k) q1[k] = q[k];
        v1 = ld3(S, kAdjV, n, i);
        w1 = ld3(S, kAdjW, n, i);
    }
    mv = mid ? vh : v1;
    mw = mid ? wh : w1;
}

}  // namespace

// Owner state of the engine <-> [29][n], one thread per (field, owner).
__device__ __forceinline__ double* owner_field(const Owners& o, int f)
{
    switch (f) {
    case 0: return o.px; case 1: return o.py; case 2: return o.pz;
    case 3: return o.qw; case 4: return o.qx; case 5: return o.qy; case 6: return o.qz;
    case 7: return o.vx; case 8: return o.vy; case 9: return o.vz;
    case 10: return o.wx; case 11: return o.wy; case 12: return o.wz;
    case 13: return o.vhx; case 14: return o.vhy; case 15: return o.vhz;
    case 16: return o.whx; case 17: return o.why; case 18: return o.whz;
    case 19: return o.hqw; case 20: return o.hqx; case 21: return o.hqy; case 22: return o.hqz;
    case 23: return o.ax; case 24: return o.ay; case 25: return o.az;
    case 26: return o.awx; case 27: return o.awy; default: return o.awz;
    }
}
__global__ void k_adj_snapshot(Owners o, double* S, const int* slot)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, f = blockIdx.y;
    const int n = o.n;
    if (i >= n) return;
    if (slot) S += (size_t)*slot * kAdjFields * n;
    S[(size_t)f * n + i] = owner_field(o, f)[i];
}
__global__ void k_adj_restore(Owners o, const double* S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, f = blockIdx.y;
    const int n = o.n;
    if (i >= n) return;
    owner_field(o, f)[i] = S[(size_t)f * n + i];
}

// Compact checkpoints of one history kind: each component keeps only its
// occupied prefix [0, hw) of slots.  Every slot at or beyond hw is empty
// (key 0, last seen -1, values 0): acquire takes the first empty slot at or
// below hw, and expire clears a slot before it lowers hw past it.  So the
// prefixes at their offsets (an exclusive scan of hw) restore the history
// exactly: the unpack writes the prefix back and clears the slots between
// the stored and the live mark.
__global__ void k_ckpt_pack(Hist<double> h, int slots, int nc, const int* off, uint64_t* key, int* last,
                            double* val)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int m = h.hw[c];
        const size_t src = (size_t)c * slots, dst = (size_t)off[c];
        for (int q = 0; q < m; ++q) {
            key[dst + q] = h.key[hslot(h, c, q)];
            last[dst + q] = h.last[hslot(h, c, q)];
            for (int a = 0; a < kHV; ++a) val[(dst + q) * kHV + a] = h.val[(src + q) * kHV + a];
        }
    }
}
__global__ void k_ckpt_unpack(Hist<double> h, int slots, int nc, const int* hw, const int* off, const uint64_t* key,
                              const int* last, const double* val)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int m = hw[c], live = h.hw[c];
        const size_t dst = (size_t)c * slots, src = (size_t)off[c];
        for (int q = 0; q < max(m, live); ++q) {
            const bool kept = q < m;
            h.key[hslot(h, c, q)] = kept ? key[src + q] : 0ull;
            h.last[hslot(h, c, q)] = kept ? last[src + q] : -1;
            for (int a = 0; a < kHV; ++a) h.val[(dst + q) * kHV + a] = kept ? val[(src + q) * kHV + a] : 0.0;
        }
        h.hw[c] = m;
    }
}

// finish^T and the owner part of forces^T for step s: S = S_s, S1 = S_{s+1},
// L = adjoint of S_{s+1} (in), Lp = adjoint of S_s (vh, wh partials out),
// P = post-advance state, T = adjoints of the post-advance state, of the
// midpoint velocities (zeroed, filled by the contact kernels), and of the
// total force and torque.  With init = 1 the step is the first evaluation
// (dt = 0, no advance, no midpoint) followed by initializeLeapfrogKernel
// (:185-210) with half step h: L is then the adjoint of S_0.  R = double:
// the FP64 map; R = float: the post-advance state and every adjoint that
// carries from step to step stay FP64, the quaternion and rotation maps'
// increments (and the world-frame spins the FP32 contact laws read) are
// FP32.
template <typename R>
__global__ void k_adj_finish(Owners o, const double* S, const double* S1, const double* L, double* Lp, double* P,
                             double* T, double dt, int init, const int* slot)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = o.n;
    if (i >= n) return;
    if (slot) {
        S += (size_t)*slot * kAdjFields * n;
        S1 = S + (size_t)kAdjFields * n;
    }
    const bool moves = !init && o.status[i] != -1;
    const bool mid = !init && o.status[i] != -1;
    D3 x1, v1, w1, mv, mw;
    double q1[4];
    post_advance(S, n, i, dt, moves, mid, x1, q1, v1, w1, mv, mw);
    st3(P, kPX, n, i, x1); st4(P, kPQ, n, i, q1); st3(P, kPV, n, i, v1); st3(P, kPW, n, i, w1);
    st3(P, kPMV, n, i, mv); st3(P, kPMW, n, i, mw);
    R qr[4];
    for (int k = 0; k < 4; ++k) qr[k] = cv<R>(q1[k]);
    const V3<R> w1r = cvt<R>(w1);
    // the world-frame spins every contact of the owner uses
    st3(P, kPEW, n, i, cvt<double>(rotq(qr, w1r))); st3(P, kPEMW, n, i, cvt<double>(rotq(qr, cvt<R>(mw))));
    // S1's finish half: the half step h = dt/2 of the finish, or the
    // leapfrog start's half step (dt holds it when init)
    const R h = cv<R>(init ? dt : 0.5 * dt);
    const double dtv = dt;  // velocity increment: the step, or the start's half step when init
    const V3<R> wh1 = cvt<R>(ld3(S1, kAdjWH, n, i));
    double lhq_d[4], lq1[4];
    R lhq[4], lp[4] = {0, 0, 0, 0}, ls[4] = {0, 0, 0, 0};
    ld4(L, kAdjHQ, n, i, lhq_d);
    for (int k = 0; k < 4; ++k) lhq[k] = cv<R>(lhq_d[k]);
    // hq1 = G(p, wh1), p = N(s), s = q1 + h G(q1, w1)
    R s[4], g[4];
    quatd(qr, w1r, g);
    for (int k = 0; k < 4; ++k) s[k] = qr[k] + g[k] * h;
    R p[4] = {s[0], s[1], s[2], s[3]};
    normq(p);
    D3 lwh1 = ld3(L, kAdjWH, n, i);
    quatd_vjp(p, wh1, lhq, lp, lwh1);
    normq_vjp(s, lp, ls);
    ld4(L, kAdjQ, n, i, lq1);
    D3 lw1 = ld3(L, kAdjW, n, i);
    for (int k = 0; k < 4; ++k) lq1[k] += cv<double>(ls[k]);
    R lsh[4];
    for (int k = 0; k < 4; ++k) lsh[k] = ls[k] * h;
    quatd_vjp(qr, w1r, lsh, lq1, lw1);
    // vh1 = vh + a1 dt (or v0 + a0 h), wh1 likewise
    const D3 lvh1 = ld3(L, kAdjVH, n, i);
    const D3 la1 = ld3(L, kAdjA, n, i) + lvh1 * dtv;
    const D3 law1 = ld3(L, kAdjAW, n, i) + lwh1 * dtv;
    D3 lv1 = ld3(L, kAdjV, n, i);
    if (init) {
        // the start adds vh0 = v0 + a0 h, wh0 = w0 + aw0 h
        lv1 = lv1 + lvh1;
        lw1 = lw1 + lwh1;
        st3(Lp, kAdjVH, n, i, z3());
        st3(Lp, kAdjWH, n, i, z3());
    } else {
        st3(Lp, kAdjVH, n, i, lvh1);
        st3(Lp, kAdjWH, n, i, lwh1);
    }
    // forces^T, owner part: a1 = F / m; Euler's equations in the body frame,
    // aw1 = (R(q1)^T tau - gyro(w1)) / I with gyro = ((Iz - Iy) wz wy,
    // (Ix - Iz) wx wz, (Iy - Ix) wy wx) (zero for isotropic inertia)
    const double m = o.mass[i], Ix = o.ix[i], Iy = o.iy[i], Iz = o.iz[i];
    const bool iso = o.iso[i] != 0;
    const D3 lF = la1 * (1.0 / m);
    const D3 aw1 = ld3(S1, kAdjAW, n, i);
    D3 tb = mk(Ix * aw1.x, Iy * aw1.y, Iz * aw1.z);
    if (!iso) tb = tb + mk((Iz - Iy) * w1.z * w1.y, (Ix - Iz) * w1.x * w1.z, (Iy - Ix) * w1.y * w1.x);
    const V3<R> tau = rotq(qr, cvt<R>(tb));
    const V3<R> ltr = mk(cv<R>(law1.x) / cv<R>(Ix), cv<R>(law1.y) / cv<R>(Iy), cv<R>(law1.z) / cv<R>(Iz));
    const D3 lt = cvt<double>(ltr);
    D3 ltau = z3();
    rotq_t_vjp(qr, tau, ltr, lq1, ltau);
    if (!iso) {
        lw1.z -= lt.x * (Iz - Iy) * w1.y; lw1.y -= lt.x * (Iz - Iy) * w1.z;
        lw1.x -= lt.y * (Ix - Iz) * w1.z; lw1.z -= lt.y * (Ix - Iz) * w1.x;
        lw1.y -= lt.z * (Iy - Ix) * w1.x; lw1.x -= lt.z * (Iy - Ix) * w1.y;
    }
    st3(T, kTX, n, i, ld3(L, kAdjX, n, i));
    st4(T, kTQ, n, i, lq1);
    st3(T, kTV, n, i, lv1);
    st3(T, kTW, n, i, lw1);
    st3(T, kTMV, n, i, z3());
    st3(T, kTMW, n, i, z3());
    st3(T, kTF, n, i, lF);
    st3(T, kTTau, n, i, ltau);
    st3(T, kTEW, n, i, z3());
    st3(T, kTEMW, n, i, z3());
}

// Material gradients of one block, by scene: a few shared rows tagged with
// their scene.  A thread adds its running sums to its scene's row when its
// scene changes and at the end; a scene that finds no row free goes straight
// to global memory.  `grads` is scene-major, [scene][3][kAdjParams], and
// `chan` selects the particle (0), wall (1) or particle-triangle (2)
// parameters.
constexpr int kGradRows = 4;
struct GradRows {
    int tag[kGradRows];
    double g[kGradRows][kAdjParams];
};
__device__ void grad_rows_init(GradRows& r)
{
    if (threadIdx.x < kGradRows) r.tag[threadIdx.x] = -1;
    if (threadIdx.x < kGradRows * kAdjParams) (&r.g[0][0])[threadIdx.x] = 0.0;
    __syncthreads();
}
__device__ void grad_add(GradRows& r, int s, const MatGrad& g, double* grads, int chan)
{
    const double gv[kAdjParams] = {g.kN, g.mu, g.logN, g.logS, g.muT, g.muR};
    int row = -1;
    for (int j = 0; j < kGradRows && row < 0; ++j) {
        const int t = atomicCAS(&r.tag[j], -1, s);  // claims a free row, or reads its scene
        if (t == -1 || t == s) row = j;
    }
    for (int f = 0; f < kAdjParams; ++f) {
        if (row >= 0) atomicAdd(&r.g[row][f], gv[f]);
        else atomicAdd(grads + ((size_t)s * 3 + chan) * kAdjParams + f, gv[f]);
    }
}
__device__ void grad_rows_flush(GradRows& r, double* grads, int chan)
{
    __syncthreads();
    if (threadIdx.x < kGradRows * kAdjParams) {
        const int j = threadIdx.x / kAdjParams, f = threadIdx.x % kAdjParams;
        if (r.tag[j] >= 0) atomicAdd(grads + ((size_t)r.tag[j] * 3 + chan) * kAdjParams + f, r.g[j][f]);
    }
}

// The entries [k, end) of a block, visited with stride `step`.  One scene:
// grid-stride over all entries.  A batch: a contiguous share of the entries
// per block, so that a thread's scene changes rarely (the entries of one
// warp's components sit together in the tape).
struct EntryRange {
    int k, end, step;
};
__device__ EntryRange entry_range(int count, int block, int blocks, int nscenes)
{
    if (nscenes == 1) return {block * (int)blockDim.x + (int)threadIdx.x, count, blocks * (int)blockDim.x};
    const int per = (count + blocks - 1) / blocks;
    const int k0 = block * per;
    return {k0 + (int)threadIdx.x, min(count, k0 + per), (int)blockDim.x};
}

template <typename R> __device__ MatGrad grad64(const MatGradT<R>& g)
{
    return MatGrad{cv<double>(g.kN), cv<double>(g.mu), cv<double>(g.logN), cv<double>(g.logS), cv<double>(g.muT),
                   cv<double>(g.muR)};
}
template <typename R> __device__ const auto& mat_of(const MatC& m, const MatF& f)
{
    if constexpr (std::is_same<R, double>::value) return m;
    else return f;
}

// Particle contact sides of one step (tape entries), reverse.  R = double:
// the FP64 map; R = float: the law's map in FP32 from FP64 differences of
// the positions and velocities (the overlap from the FP64 difference of
// squares), the adjoints scattered into the owners in FP64.
template <typename R>
__device__ void adj_pp(Comps c, Owners o, const SceneC* __restrict__ sc, StepTape tp, int count, const double* P,
                       double* T, double* lhist, double dt_eff, double* grads, int block, int blocks, int nscenes,
                       GradRows& rows)
{
    const int n = o.n;
    tp = tape_at(tp);
    if (count < 0) count = min(*tp.pp_count, tp.pp_cap);
    grad_rows_init(rows);
    MatGradT<R> gsum = {0, 0, 0, 0, 0, 0};
    int cur = -1;  // the scene gsum belongs to
    const EntryRange er = entry_range(count, block, blocks, nscenes);
    for (int k = er.k; k < er.end; k += er.step) {
        const int4 e = tp.pp[k];
        const int i = e.x, j = e.y;
        const int si = nscenes == 1 ? 0 : o.scene[i];
        if (si != cur) {
            if (cur >= 0) grad_add(rows, cur, grad64(gsum), grads, 0);
            gsum = MatGradT<R>{0, 0, 0, 0, 0, 0};
            cur = si;
        }
        const auto& m = mat_of<R>(sc[si].pp, sc[si].ppf);
        D3 xi = ld3(P, kPX, n, i), xj = ld3(P, kPX, n, j);
        const D3 vi = ld3(P, kPV, n, i), vj = ld3(P, kPV, n, j);
        const D3 mvi = ld3(P, kPMV, n, i), mvj = ld3(P, kPMV, n, j);
        const D3 delta = xj - xi;
        const double ri = c.radius[i], rj = c.radius[j];
        PPInT<R> in;
        in.delta = cvt<R>(delta);
        if constexpr (!std::is_same<R, double>::value) {
            const double rs = ri + rj, d2 = dot(delta, delta);
            in.depth = cv<R>(rs * rs - d2) / (cv<R>(rs) + sqrt(dot(in.delta, in.delta)));
        }
        in.ri = cv<R>(ri); in.rj = cv<R>(rj); in.mi = cv<R>(o.mass[i]); in.mj = cv<R>(o.mass[j]);
        in.erv = cvt<R>(vj - vi);
        in.mrv = cvt<R>(mvj - mvi);
        in.ewi = cvt<R>(ld3(P, kPEW, n, i)); in.ewj = cvt<R>(ld3(P, kPEW, n, j));
        in.mwi = cvt<R>(ld3(P, kPEMW, n, i)); in.mwj = cvt<R>(ld3(P, kPEMW, n, j));
        for (int a = 0; a < 9; ++a) in.h[a] = cv<R>(tp.pp_h[(size_t)k * kHV + a]);
        double* lh = lhist + (size_t)e.z * kHV;
        R lho[9];
        for (int a = 0; a < 9; ++a) lho[a] = cv<R>(lh[a]);
        PPAdjT<R> ad;
        ad.delta = ad.erv = ad.mrv = ad.ewi = ad.ewj = ad.mwi = ad.mwj = zr<R>();
        for (int a = 0; a < 9; ++a) ad.h[a] = R(0);
        pp_law_vjp(m, cv<R>(dt_eff), in, cvt<R>(ld3(T, kTF, n, i)), cvt<R>(ld3(T, kTTau, n, i)), lho, ad, gsum);
        for (int a = 0; a < 9; ++a) lh[a] = e.w ? 0.0 : cv<double>(ad.h[a]);
        const D3 adelta = cvt<double>(ad.delta), aerv = cvt<double>(ad.erv), amrv = cvt<double>(ad.mrv);
        add3(T, kTX, n, j, adelta);
        add3(T, kTX, n, i, adelta * -1.0);
        add3(T, kTV, n, j, aerv);
        add3(T, kTV, n, i, aerv * -1.0);
        add3(T, kTMV, n, j, amrv);
        add3(T, kTMV, n, i, amrv * -1.0);
        add3(T, kTEW, n, i, cvt<double>(ad.ewi));
        add3(T, kTEW, n, j, cvt<double>(ad.ewj));
        add3(T, kTEMW, n, i, cvt<double>(ad.mwi));
        add3(T, kTEMW, n, j, cvt<double>(ad.mwj));
    }
    if (cur >= 0) grad_add(rows, cur, grad64(gsum), grads, 0);
    grad_rows_flush(rows, grads, 0);
}

template <typename R>
__device__ void pw_one(const Comps& c, const Owners& o, const SceneC& S, const Walls& walls, const StepTape& tp, int k,
                       const double* P, double* T, double* lhist, double dt_eff, MatGradT<R>& g)
{
    const int n = o.n;
    const int4 e = tp.pw[k];
    const int i = e.x;
    const int wg = S.wall_begin + e.y;
    const D3 out = mk(walls.n[3 * wg], walls.n[3 * wg + 1], walls.n[3 * wg + 2]);
    const D3 org = mk(walls.o[3 * wg], walls.o[3 * wg + 1], walls.o[3 * wg + 2]);
    const D3 x1 = ld3(P, kPX, n, i), v1 = ld3(P, kPV, n, i);
    const double r = c.radius[i];
    const double depth = r - dot(x1 - org, out);
    const D3 om = ld3(P, kPEW, n, i);
    R hin[9], lho[9];
    for (int a = 0; a < 9; ++a) hin[a] = cv<R>(tp.pw_h[(size_t)k * kHV + a]);
    double* lh = lhist + (size_t)e.z * kHV;
    for (int a = 0; a < 9; ++a) lho[a] = cv<R>(lh[a]);
    PWAdjT<R> ad;
    ad.p = ad.vel = ad.om = zr<R>();
    for (int a = 0; a < 9; ++a) ad.h[a] = R(0);
    pw_law_vjp(mat_of<R>(S.pw, S.pwf), cv<R>(dt_eff), cvt<R>(out), cv<R>(depth), cv<R>(r), cv<R>(o.mass[i]),
               cvt<R>(v1), cvt<R>(om), hin, cvt<R>(ld3(T, kTF, n, i)), cvt<R>(ld3(T, kTTau, n, i)), lho, ad, g);
    for (int a = 0; a < 9; ++a) lh[a] = e.w ? 0.0 : cv<double>(ad.h[a]);
    add3(T, kTX, n, i, cvt<double>(ad.p));
    add3(T, kTV, n, i, cvt<double>(ad.vel));
    add3(T, kTEW, n, i, cvt<double>(ad.om));
}

// Wall contacts of one step (tape entries), reverse.
template <typename R>
__device__ void adj_pw(Comps c, Owners o, const SceneC* __restrict__ sc, Walls walls, StepTape tp, int count,
                       const double* P, double* T, double* lhist, double dt_eff, double* grads, int block, int blocks,
                       int nscenes, GradRows& rows)
{
    tp = tape_at(tp);
    if (count < 0) count = min(*tp.pw_count, tp.pw_cap);
    grad_rows_init(rows);
    MatGradT<R> g = {0, 0, 0, 0, 0, 0};
    int cur = -1;
    const EntryRange er = entry_range(count, block, blocks, nscenes);
    for (int k = er.k; k < er.end; k += er.step) {
        const int si = nscenes == 1 ? 0 : o.scene[tp.pw[k].x];
        if (si != cur) {
            if (cur >= 0) grad_add(rows, cur, grad64(g), grads, 1);
            g = MatGradT<R>{0, 0, 0, 0, 0, 0};
            cur = si;
        }
        MatGradT<R> gk = {0, 0, 0, 0, 0, 0};
        pw_one<R>(c, o, sc[si], walls, tp, k, P, T, lhist, dt_eff, gk);
        g.kN += gk.kN; g.mu += gk.mu; g.logN += gk.logN; g.logS += gk.logS; g.muT += gk.muT; g.muR += gk.muR;
    }
    if (cur >= 0) grad_add(rows, cur, grad64(g), grads, 1);
    grad_rows_flush(rows, grads, 1);
}

// Particle and wall contacts of one step in one launch: blocks [0, bpp) take
// the particle entries, the rest the wall entries.  Each entry's reverse law
// is a long serial FP64 chain, and a warp issues one FP64 instruction per
// about 68 cycles whatever its neighbours do, so with few contacts the two
// sets cost their longer chain instead of the sum of both.  The FP32 form is
// compiled for 4 resident blocks (128 registers; the compiler's own choice
// was 168, 3 blocks): the 64-scene batch's backward run 0.299 -> 0.293 s.
template <typename R>
__global__ void __launch_bounds__(128, sizeof(R) == sizeof(float) ? 4 : 1) k_adj_contacts(Comps c, Owners o, const SceneC* __restrict__ sc, Walls walls,
                                                      StepTape tp, int npp, int npw, int bpp, const double* P, double* T,
                                                      double* lh_pp, double* lh_pw, double dt_eff, double* grads,
                                                      int nscenes)
{
    __shared__ GradRows rows;
    if ((int)blockIdx.x < bpp)
        adj_pp<R>(c, o, sc, tp, npp, P, T, lh_pp, dt_eff, grads, blockIdx.x, bpp, nscenes, rows);
    else
        adj_pw<R>(c, o, sc, walls, tp, npw, P, T, lh_pw, dt_eff, grads, blockIdx.x - bpp, gridDim.x - bpp, nscenes,
                  rows);
}


// Particle-body manifolds of one step (tape entries), reverse: one thread
// per manifold.  The sphere's adjoints go to T like a wall contact's; the
// body's pose adjoints (centre, orientation, velocity, spin) to its row of
// the body adjoints; the adjoint of the body's reaction load comes from
// the row's kBlF (the half update's reverse, run before this kernel).
__device__ __forceinline__ int adj_global_step(const int* base, const int* slot)
{
    return (base ? *base : 0) + (slot ? *slot : 0);
}
__global__ void __launch_bounds__(64) k_adj_pt(Comps c, Owners o, const SceneC* __restrict__ sc, StepTape tp, int count,
                                               const double* P, double* T, double* lhist, AdjBodies ab, double dt_eff,
                                               double* grads, int nscenes)
{
    __shared__ GradRows rows;
    const int n = o.n;
    const int g = adj_global_step(ab.base, tp.slot);
    tp = tape_at(tp);
    if (count < 0) count = min(*tp.pb_count, tp.pb_cap);
    grad_rows_init(rows);
    MatGrad gs = {0, 0, 0, 0, 0, 0};
    int cur = -1;
    const EntryRange er = entry_range(count, blockIdx.x, gridDim.x, nscenes);
    for (int k = er.k; k < er.end; k += er.step) {
        const int4 e = tp.pb[k];
        const int i = e.x, b = e.y;
        const int si = nscenes == 1 ? 0 : o.scene[i];
        if (si != cur) {
            if (cur >= 0) grad_add(rows, cur, gs, grads, 2);
            gs = MatGrad{0, 0, 0, 0, 0, 0};
            cur = si;
        }
        const double* rec = ab.rec + ((size_t)g * ab.nb + b) * kBR;
        PTIn in;
        in.p = ld3(P, kPX, n, i); in.ev = ld3(P, kPV, n, i); in.mv = ld3(P, kPMV, n, i);
        in.ew = ld3(P, kPEW, n, i); in.mw = ld3(P, kPEMW, n, i);
        in.rad = c.radius[i]; in.mass = o.mass[i];
        in.c = ldv3(rec, kBrC); in.V = ldv3(rec, kBrV); in.w = ldv3(rec, kBrW);
        for (int q = 0; q < 4; ++q) in.q[q] = rec[kBrQ + q];
        const int* tl = tp.pb_tri + (size_t)k * kPbTri;
        in.ntri = min(tl[0], kPbTris);
        for (int t = 0; t < in.ntri; ++t) in.L[t] = ab.local + 15 * (size_t)tl[1 + t];
        for (int a = 0; a < 9; ++a) in.h[a] = tp.pb_h[(size_t)k * kHV + a];
        double* lh = lhist + (size_t)e.z * kHV;
        double lho[9];
        for (int a = 0; a < 9; ++a) lho[a] = lh[a];
        PTAdj ad;
        ad.p = ad.ev = ad.mv = ad.ew = ad.mw = ad.c = ad.V = ad.w = z3();
        for (int q = 0; q < 4; ++q) ad.q[q] = 0.0;
        for (int a = 0; a < 9; ++a) ad.h[a] = 0.0;
        double* Lb = ab.L + (size_t)b * kBL;
        pt_manifold_vjp(sc[si].pt, dt_eff, in, ld3(T, kTF, n, i), ld3(T, kTTau, n, i), ldv3(Lb, kBlF),
                        ldv3(Lb, kBlF + 3), lho, ad, gs);
        for (int a = 0; a < 9; ++a) lh[a] = e.w ? 0.0 : ad.h[a];
        add3(T, kTX, n, i, ad.p);
        add3(T, kTV, n, i, ad.ev);
        add3(T, kTMV, n, i, ad.mv);
        add3(T, kTEW, n, i, ad.ew);
        add3(T, kTEMW, n, i, ad.mw);
        const double pose[13] = {ad.c.x, ad.c.y, ad.c.z, ad.q[0], ad.q[1], ad.q[2], ad.q[3],
                                 ad.V.x, ad.V.y, ad.V.z, ad.w.x, ad.w.y, ad.w.z};
        for (int f = 0; f < 13; ++f) atomicAdd(Lb + kBlC + f, pose[f]);
    }
    if (cur >= 0) grad_add(rows, cur, gs, grads, 2);
    grad_rows_flush(rows, grads, 2);
}

// The body leapfrog's reverse, one thread per body (dynamic bodies only:
// the others follow their prescribed or fixed motion and carry no
// adjoint).  Part A: the half update of the step (before the contacts'
// reverse, which reads the loads' adjoint).  Part C: the position update
// into the step, from the previous step's record.
__global__ void k_adj_body_a(AdjBodies ab, const int* slot, int first)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= ab.nb) return;
    double* Lb = ab.L + (size_t)b * kBL;
    const double* cst = ab.cst + 5 * (size_t)b;
    if (cst[4] != 0.0) {
        for (int f = 0; f < kBL; ++f) Lb[f] = 0.0;
        return;
    }
    const int g = adj_global_step(ab.base, slot);
    body_half_vjp(ab.rec + ((size_t)g * ab.nb + b) * kBR, cst, ab.dt, first != 0, Lb);
}
__global__ void k_adj_body_c(AdjBodies ab, const int* slot)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= ab.nb) return;
    double* Lb = ab.L + (size_t)b * kBL;
    if (ab.cst[5 * (size_t)b + 4] != 0.0) {
        for (int f = 0; f < kBL; ++f) Lb[f] = 0.0;
        return;
    }
    const int g = adj_global_step(ab.base, slot);
    body_pos_vjp(ab.rec + ((size_t)(g - 1) * ab.nb + b) * kBR, ab.dt, Lb);
}
__global__ void k_adj_body_pose(Bodies bd, const double* rec, const int* base, const int* slot)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bd.nb) return;
    const double* r = rec + ((size_t)adj_global_step(base, slot) * bd.nb + b) * kBR;
    for (int a = 0; a < 3; ++a) {
        bd.c[3 * b + a] = r[kBrC + a];
        bd.v[3 * b + a] = r[kBrV + a];
        bd.w[3 * b + a] = r[kBrW + a];
    }
    for (int q = 0; q < 4; ++q) bd.q[4 * b + q] = r[kBrQ + q];
}
__global__ void k_set_int(int* p, int v) { *p = v; }

// advance^T: T (complete) and the vh, wh partials of Lp -> Lp = adjoint of
// S_s.  With init = 1 (the first evaluation, no advance): Lp = adjoint of
// the initial x, q, v, w.  R as k_adj_finish: the rotations' increments in
// R, the normalisation's map of the carried quaternion adjoint in FP64.
template <typename R>
__global__ void k_adj_advance(Owners o, const double* S, const double* P, const double* T, double* Lp, double dt,
                              int init, const int* slot)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = o.n;
    if (i >= n) return;
    if (slot) S += (size_t)*slot * kAdjFields * n;
    const D3 lx1 = ld3(T, kTX, n, i), lv1 = ld3(T, kTV, n, i);
    D3 lw1 = ld3(T, kTW, n, i);
    const D3 lmv = ld3(T, kTMV, n, i);
    D3 lmw = ld3(T, kTMW, n, i);
    double lq1[4];
    ld4(T, kTQ, n, i, lq1);
    {
        // the contacts' adjoints of the world-frame spins R(q1) w1 and
        // R(q1) w_mid, to the quaternion and the body-frame spins
        double q1[4];
        ld4(P, kPQ, n, i, q1);
        R qr[4];
        for (int k = 0; k < 4; ++k) qr[k] = cv<R>(q1[k]);
        rotq_vjp(qr, cvt<R>(ld3(P, kPW, n, i)), cvt<R>(ld3(T, kTEW, n, i)), lq1, lw1);
        rotq_vjp(qr, cvt<R>(ld3(P, kPMW, n, i)), cvt<R>(ld3(T, kTEMW, n, i)), lq1, lmw);
    }
    const bool moves = !init && o.status[i] != -1;
    double zero4[4] = {0, 0, 0, 0};
    if (!moves) {
        // no advance and no midpoint: the laws saw x, q, v, w themselves
        st3(Lp, kAdjX, n, i, lx1);
        st4(Lp, kAdjQ, n, i, lq1);
        st3(Lp, kAdjV, n, i, lv1 + lmv);
        st3(Lp, kAdjW, n, i, lw1 + lmw);
        if (!init) {
            st3(Lp, kAdjVH, n, i, ld3(Lp, kAdjVH, n, i));
            st3(Lp, kAdjWH, n, i, ld3(Lp, kAdjWH, n, i));
        }
        st4(Lp, kAdjHQ, n, i, zero4);
        st3(Lp, kAdjA, n, i, z3());
        st3(Lp, kAdjAW, n, i, z3());
        return;
    }
    double q[4], hq[4];
    ld4(S, kAdjQ, n, i, q);
    ld4(S, kAdjHQ, n, i, hq);
    double r[4], lr[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k) r[k] = q[k] + hq[k] * dt;
    normq_vjp(r, lq1, lr);
    D3 lvh = ld3(Lp, kAdjVH, n, i) + lmv + lx1 * dt + lv1;
    D3 lwh = ld3(Lp, kAdjWH, n, i) + lmw + lw1;
    st3(Lp, kAdjX, n, i, lx1);
    st4(Lp, kAdjQ, n, i, lr);
    double lhq[4];
    for (int k = 0; k < 4; ++k) lhq[k] = lr[k] * dt;
    st4(Lp, kAdjHQ, n, i, lhq);
    st3(Lp, kAdjV, n, i, z3());
    st3(Lp, kAdjW, n, i, z3());
    st3(Lp, kAdjVH, n, i, lvh);
    st3(Lp, kAdjWH, n, i, lwh);
    st3(Lp, kAdjA, n, i, lv1 * (0.5 * dt));
    st3(Lp, kAdjAW, n, i, lw1 * (0.5 * dt));
}

// ---------------------------------------------------------- launchers
void launch_adj_snapshot(const Owners& o, double* S, cudaStream_t s, const int* slot)
{
    if (o.n > 0) k_adj_snapshot<<<dim3(nblocks(o.n, 256), kAdjFields), 256, 0, s>>>(o, S, slot);
}
void launch_adj_restore(const Owners& o, const double* S, cudaStream_t s)
{
    if (o.n > 0) k_adj_restore<<<dim3(nblocks(o.n, 256), kAdjFields), 256, 0, s>>>(o, S);
}
void launch_ckpt_pack(const Hist<double>& h, int slots, int nc, const int* off, uint64_t* key, int* last, double* val,
                      int sm_count, cudaStream_t s)
{
    if (nc > 0) k_ckpt_pack<<<std::max(1, std::min(nblocks(nc, 256), sm_count * 8)), 256, 0, s>>>(h, slots, nc, off, key,
                                                                                                   last, val);
}
void launch_ckpt_unpack(const Hist<double>& h, int slots, int nc, const int* hw, const int* off, const uint64_t* key,
                        const int* last, const double* val, int sm_count, cudaStream_t s)
{
    if (nc > 0)
        k_ckpt_unpack<<<std::max(1, std::min(nblocks(nc, 256), sm_count * 8)), 256, 0, s>>>(h, slots, nc, hw, off, key,
                                                                                             last, val);
}
void launch_adj_step(const Comps& c, const Owners& o, const SceneC* sc, const Walls& w, const StepTape& tp, int npp,
                     int npw, int npb, const double* S, const double* S1, const double* L, double* Lp, double* P,
                     double* T, double* lh_pp, double* lh_pw, double* lh_pb, const AdjBodies& ab, double dt,
                     double dt_eff, int init, double* grads, int nscenes, int sm_count, cudaStream_t s,
                     cudaStream_t s2, cudaEvent_t* ev, bool fp32)
{
    if (o.n <= 0) return;
    // device counts: S, S1 at the tape's slot, fixed grid-stride grids
    const int* slot = (npp < 0 || npw < 0) ? tp.slot : nullptr;
    const bool bodies = ab.nb > 0 && tp.pb;
    // with bodies and a second stream, a DAG: the body leapfrog's reverse
    // and the manifolds' run beside the owners' finish and the contacts
    // (each a chain of dependent FP64 work on a few threads)
    const bool fork = bodies && s2 && ev;
    cudaStream_t sb = fork ? s2 : s;
    if (fork) {
        cudaEventRecord(ev[0], s);
        cudaStreamWaitEvent(s2, ev[0], 0);
    }
    if (bodies) k_adj_body_a<<<nblocks(ab.nb, 32), 32, 0, sb>>>(ab, slot, init);
    if (fp32)
        k_adj_finish<float><<<nblocks(o.n, 256), 256, 0, s>>>(o, S, S1, L, Lp, P, T, dt, init, slot);
    else
        k_adj_finish<double><<<nblocks(o.n, 256), 256, 0, s>>>(o, S, S1, L, Lp, P, T, dt, init, slot);
    if (fork) {
        cudaEventRecord(ev[1], s);
        cudaStreamWaitEvent(s2, ev[1], 0);
    }
    if (bodies) {
        const int bpb = npb < 0 ? sm_count * 2 : min(nblocks(npb, 64), sm_count * 2);
        if (bpb > 0) k_adj_pt<<<bpb, 64, 0, sb>>>(c, o, sc, tp, npb, P, T, lh_pb, ab, dt_eff, grads, nscenes);
        if (!init) k_adj_body_c<<<nblocks(ab.nb, 32), 32, 0, sb>>>(ab, slot);
    }
    const int bpp = npp < 0 ? sm_count * 8 : min(nblocks(npp, 128), sm_count * 8);
    const int bpw = npw < 0 ? sm_count * 2 : min(nblocks(npw, 128), sm_count * 2);
    if (bpp + bpw > 0) {
        if (fp32)
            k_adj_contacts<float><<<bpp + bpw, 128, 0, s>>>(c, o, sc, w, tp, npp, npw, bpp, P, T, lh_pp, lh_pw, dt_eff,
                                                            grads, nscenes);
        else
            k_adj_contacts<double><<<bpp + bpw, 128, 0, s>>>(c, o, sc, w, tp, npp, npw, bpp, P, T, lh_pp, lh_pw, dt_eff,
                                                             grads, nscenes);
    }
    if (fork) {
        cudaEventRecord(ev[2], s2);
        cudaStreamWaitEvent(s, ev[2], 0);
    }
    if (fp32)
        k_adj_advance<float><<<nblocks(o.n, 256), 256, 0, s>>>(o, S, P, T, Lp, dt, init, slot);
    else
        k_adj_advance<double><<<nblocks(o.n, 256), 256, 0, s>>>(o, S, P, T, Lp, dt, init, slot);
}
void launch_adj_body_pose(const Bodies& b, const double* rec, const int* base, const int* slot, cudaStream_t s)
{
    if (b.nb > 0) k_adj_body_pose<<<nblocks(b.nb, 32), 32, 0, s>>>(b, rec, base, slot);
}
void launch_set_int(int* p, int v, cudaStream_t s) { k_set_int<<<1, 1, 0, s>>>(p, v); }

__global__ void k_adj_slot_add(int* slot, int delta) { *slot += delta; }
__global__ void k_adj_tape_begin(int* pw_count, int* pb_count, const int* slot)
{
    pw_count[*slot] = 0;
    if (pb_count) pb_count[*slot] = 0;
}
__global__ void k_adj_tape_end(int* pp_count, const int* ct_total, int* slot)
{
    pp_count[*slot] = *ct_total;
    *slot += 1;
}

void launch_adj_slot_add(int* slot, int delta, cudaStream_t s) { k_adj_slot_add<<<1, 1, 0, s>>>(slot, delta); }
void launch_adj_tape_begin(int* pw_count, int* pb_count, const int* slot, cudaStream_t s)
{
    k_adj_tape_begin<<<1, 1, 0, s>>>(pw_count, pb_count, slot);
}
void launch_adj_tape_end(int* pp_count, const int* ct_total, int* slot, cudaStream_t s)
{
    k_adj_tape_end<<<1, 1, 0, s>>>(pp_count, ct_total, slot);
}

}  // namespace demgb
