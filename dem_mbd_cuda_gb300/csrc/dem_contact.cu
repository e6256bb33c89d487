// dem_contact.cu -- contact pipeline of one force evaluation.
//
// The reference evaluates everything for one owner in one thread
// (computeContactsKernel, src/cuda/cuda_contact_backend.cu:1065-1221): walls,
// a 27-cell sweep with binary searches and the full FP64 particle law inline,
// then the particle-triangle manifold.  Here the work is split so the
// expensive law runs without warp divergence:
//   gather      packed sorted rows of every component (cell order)
//   broadphase  one thread per component: history expiry, wall law, 27-cell
//               sweep over the cell start table with an FP32 cell-relative
//               prefilter and the exact FP64 overlap test, history slot
//               acquisition in sweep order, append to a flat contact list
//   pp law      one thread per contact (T = double or float)
//   pt          one thread per component whose cell holds triangles: the
//               reference's per-body manifold, then the per-triangle loads
//   owner sum   per owner, contacts summed in the reference's sweep order,
//               total force and the acceleration / Euler update fused
//   body reduce deterministic two-level reduction of the body loads
#include "dem_kernels.cuh"

#include <algorithm>

#include <climits>

namespace demgb {

namespace {

__device__ __forceinline__ int warp_sum(int v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_maxi(int v)
{
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ int block_exclusive_scan_c(int v, int& total)
{
    __shared__ int warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < nw ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    total = warp_sums[nw - 1];
    const int base = wid > 0 ? warp_sums[wid - 1] : 0;
    __syncthreads();
    return base + x - v;
}

// Block-aggregated counter updates (sum / max).
__device__ void block_add(int* dst, int v)
{
    const int s = warp_sum(v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst, s);
}
__device__ void block_max(int* dst, int v)
{
    const int s = warp_maxi(v);
    if ((threadIdx.x & 31) == 0 && s > 0) atomicMax(dst, s);
}

// One history slot <-> registers (h[0..8]; the padding is written as 0).
__device__ __forceinline__ void hv_load(const float* p, float* h)
{
    const float4* q = reinterpret_cast<const float4*>(p);
    const float4 a = q[0], b = q[1], c = q[2];
    h[0] = a.x; h[1] = a.y; h[2] = a.z; h[3] = a.w;
    h[4] = b.x; h[5] = b.y; h[6] = b.z; h[7] = b.w;
    h[8] = c.x;
}
__device__ __forceinline__ void hv_store(float* p, const float* h)
{
    float4* q = reinterpret_cast<float4*>(p);
    q[0] = make_float4(h[0], h[1], h[2], h[3]);
    q[1] = make_float4(h[4], h[5], h[6], h[7]);
    q[2] = make_float4(h[8], 0.f, 0.f, 0.f);
}
__device__ __forceinline__ void hv_load(const double* p, double* h)
{
    const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double2 v = q[k];
        h[2 * k] = v.x; h[2 * k + 1] = v.y;
    }
    h[8] = q[4].x;
}
__device__ __forceinline__ void hv_store(double* p, const double* h)
{
    double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = make_double2(h[2 * k], h[2 * k + 1]);
    q[4] = make_double2(h[8], 0.0);
}
template <typename T> __device__ __forceinline__ void zero_hv(T* v)
{
    T z[9] = {};
    hv_store(v, z);
}

// The material constants a law of precision T reads.
template <typename T> __device__ __forceinline__ const auto& mat(const MatC& d, const MatF& f)
{
    if constexpr (sizeof(T) == sizeof(double)) return d;
    else return f;
}

// Read-only load of a 32-byte record.
__device__ __forceinline__ D4 ldg_d4(const D4* p)
{
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    D4 v;
    v.x = a.x; v.y = a.y; v.z = b.x; v.w = b.y;
    return v;
}

// expireHistory (:217-229) over the occupied prefix [0, hw).  Ahead: the
// first two keys and last-seen steps load beside the high-water mark, not
// after it (for the particle slots, which nearly every component uses;
// every kind has at least two slots).
template <bool Ahead, typename T> __device__ void expire(Hist<T> h, int slots, int c, int step)
{
    const size_t base = (size_t)c * slots;
    uint64_t k0 = 0, k1 = 0;
    int l0 = 0, l1 = 0;
    if (Ahead) {
        k0 = h.key[hslot(h, c, 0)];
        k1 = h.key[hslot(h, c, 1)];
        l0 = h.last[hslot(h, c, 0)];
        l1 = h.last[hslot(h, c, 1)];
    }
    const int hw = h.hw[c];
    int nhw = 0;
    for (int s = 0; s < hw; ++s) {
        const uint64_t key = Ahead && s == 0 ? k0 : Ahead && s == 1 ? k1 : h.key[hslot(h, c, s)];
        if (key != 0) {
            const int last = Ahead && s == 0 ? l0 : Ahead && s == 1 ? l1 : h.last[hslot(h, c, s)];
            if (last < step - 1) {
                h.key[hslot(h, c, s)] = 0;
                h.last[hslot(h, c, s)] = -1;
                zero_hv(h.val + (base + s) * kHV);
            } else {
                nhw = s + 1;
            }
        }
    }
    if (nhw != hw) h.hw[c] = nhw;
}

// acquireHistorySlot (:190-215): the matching key, else the first empty slot.
// Returns the slot index within the component, -1 on overflow.
template <typename T>
__device__ int acquire(Hist<T> h, int slots, int c, uint64_t key, int step, int& hw, int& high, bool* fresh = nullptr)
{
    if (fresh) *fresh = false;
    const size_t base = (size_t)c * slots;
    int empty = -1;
    for (int s = 0; s < hw; ++s) {
        const uint64_t k = h.key[hslot(h, c, s)];
        if (k == key) {
            h.last[hslot(h, c, s)] = step;
            high = max(high, s + 1);
            return s;
        }
        if (k == 0 && empty < 0) empty = s;
    }
    if (empty < 0) {
        if (hw >= slots) return -1;
        empty = hw;
    }
    h.key[hslot(h, c, empty)] = key;
    h.last[hslot(h, c, empty)] = step;
    zero_hv(h.val + (base + empty) * kHV);
    if (fresh) *fresh = true;
    if (empty + 1 > hw) hw = empty + 1;
    high = max(high, empty + 1);
    return empty;
}

__device__ __forceinline__ V3<double> d3(D4 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ D4 d4(double x, double y, double z, double w) { return D4{x, y, z, w}; }
__device__ __forceinline__ V3<float> f3(float4 v) { return {v.x, v.y, v.z}; }

// Quat2IvDCM rotation in FP32 (mixed form only).
__device__ __forceinline__ V3<float> rot_ivf(float qw, float qx, float qy, float qz, V3<float> v)
{
    return {(1.f - 2.f * (qy * qy + qz * qz)) * v.x + 2.f * (qx * qy - qw * qz) * v.y + 2.f * (qx * qz + qw * qy) * v.z,
            2.f * (qx * qy + qw * qz) * v.x + (1.f - 2.f * (qx * qx + qz * qz)) * v.y + 2.f * (qy * qz - qw * qx) * v.z,
            2.f * (qx * qz - qw * qy) * v.x + 2.f * (qy * qz + qw * qx) * v.y + (1.f - 2.f * (qx * qx + qy * qy)) * v.z};
}

// ------------------------------------------------------------------ gather
// The records in sorted order, in two parts: the geometry (positions,
// cells, indices: all the sweep reads, available once the positions are)
// and the velocities (after the rotational advance).
__global__ void k_gather_geom(Comps c, Owners o, Grid g, Recs r, Counters k)
{
    const int nvalid = *g.nvalid;
    const int step = k.nl_on ? *k.step : 0;
    int movers = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nvalid; t += gridDim.x * blockDim.x) {
        const int ci = g.sorted_id[t];
        const int w = c.owner[ci];
        const double x = c.x[ci], y = c.y[ci], z = c.z[ci], rad = c.radius[ci];
        r.pos[t] = d4(x, y, z, rad);
        if (r.off) r.off[t] = d4(c.ox[ci], c.oy[ci], c.oz[ci], 0.0);
        int cx, cy, cz;
        unpack_cell(g.ckey[ci], cx, cy, cz);
        const int s = o.scene[w];
        r.meta[t] = make_int4(ci, w, c.cid[ci], s);
        r.cell[t] = make_int4(cx, cy, cz, g.clin[ci]);
        const double mesh = g.sc[s].mesh;
        r.relf[t] = make_float4(f32_rn(__fma_rn(-(double)cx, mesh, x)), f32_rn(__fma_rn(-(double)cy, mesh, y)),
                                f32_rn(__fma_rn(-(double)cz, mesh, z)), f32_rn(rad));
        if (k.nl_on) {
            const double* xr = k.nl_xref + 3 * (size_t)ci;
            const double dx = x - xr[0], dy = y - xr[1], dz = z - xr[2];
            if (dx * dx + dy * dy + dz * dz > g.sc[s].nl_half2) {
                // a mover (more than half the skin since the lists' build)
                // marks the up to 27 cells around its own for this step
                const int* lay = g.scene_layout + 8 * s;
                const int z0 = max(cz - 1, lay[2]), z1 = min(cz + 1, lay[2] + lay[5] - 1);
                for (int nx = max(cx - 1, lay[0]); nx <= min(cx + 1, lay[0] + lay[3] - 1); ++nx)
                    for (int ny = max(cy - 1, lay[1]); ny <= min(cy + 1, lay[1] + lay[4] - 1); ++ny) {
                        const int row = lay[6] + ((nx - lay[0]) * lay[4] + (ny - lay[1])) * lay[5] - lay[2];
                        for (int nz = z0; nz <= z1; ++nz) k.nl_hot[row + nz] = step;
                    }
                ++movers;
            }
        }
    }
    // beyond the limit every list is rebuilt this step
    for (int o2 = 16; o2 > 0; o2 >>= 1) movers += __shfl_xor_sync(0xffffffffu, movers, o2);
    if (movers && (threadIdx.x & 31) == 0) {
        const int before = atomicAdd(k.nl_flag + 3, movers);
        if (before + movers > k.nl_limit) k.nl_flag[0] = 1;
    }
}

template <typename T> __global__ void k_gather_vel(Comps c, Owners o, Grid g, Recs r, double dt_eff)
{
    const int nvalid = *g.nvalid;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nvalid; t += gridDim.x * blockDim.x) {
        const int ci = g.sorted_id[t];
        const int w = c.owner[ci];
        const double vx = c.vx[ci], vy = c.vy[ci], vz = c.vz[ci];
        const bool mid = dt_eff > 0.0 && o.status[w] != -1;
        if constexpr (sizeof(T) == sizeof(double)) {
            r.v[t] = d4(vx, vy, vz, o.mass[w]);
            r.vm[t] = mid ? d4(c.vhx[ci], c.vhy[ci], c.vhz[ci], 0.0) : d4(vx, vy, vz, 0.0);
            const double qw = o.qw[w], qx = o.qx[w], qy = o.qy[w], qz = o.qz[w];
            const V3<double> ew = rot_iv(qw, qx, qy, qz, mk(o.wx[w], o.wy[w], o.wz[w]));
            r.w[t] = d4(ew.x, ew.y, ew.z, 0.0);
            const V3<double> mw = mid ? rot_iv(qw, qx, qy, qz, mk(o.whx[w], o.why[w], o.whz[w])) : ew;
            r.wm[t] = d4(mw.x, mw.y, mw.z, 0.0);
        } else {
            // mixed form: FP32 rows; the world-frame rotation of omega is part
            // of the per-contact FP32 arithmetic.
            const float fvx = f32_rn(vx), fvy = f32_rn(vy), fvz = f32_rn(vz);
            r.vf[t] = make_float4(fvx, fvy, fvz, f32_rn(o.mass[w]));
            r.vmf[t] = mid ? make_float4(f32_rn(c.vhx[ci]), f32_rn(c.vhy[ci]), f32_rn(c.vhz[ci]), 0.f)
                           : make_float4(fvx, fvy, fvz, 0.f);
            const float qw = f32_rn(o.qw[w]), qx = f32_rn(o.qx[w]), qy = f32_rn(o.qy[w]), qz = f32_rn(o.qz[w]);
            const V3<float> ew = rot_ivf(qw, qx, qy, qz, mk(f32_rn(o.wx[w]), f32_rn(o.wy[w]), f32_rn(o.wz[w])));
            r.wf[t] = make_float4(ew.x, ew.y, ew.z, 0.f);
            const V3<float> mw =
                mid ? rot_ivf(qw, qx, qy, qz, mk(f32_rn(o.whx[w]), f32_rn(o.why[w]), f32_rn(o.whz[w]))) : ew;
            r.wmf[t] = make_float4(mw.x, mw.y, mw.z, 0.f);
        }
    }
}

// ------------------------------------------------------ expiry and walls
// wallContact (:975-1063) for wall wl of the component's scene: the exact
// FP64 depth, slot acquisition and the wall law; the load is added to wF/wT.
template <typename T>
__device__ __noinline__ void wall_contact(const Comps& c, const Owners& o, const SceneC& S, const Walls& walls,
                                          Hist<T> hw, int ci, int w, int wl, V3<double> p, double rad, int step,
                                          double dt_eff, int& whw, int& bhigh, int& bover, V3<double>& wF,
                                          V3<double>& wT, const StepTape& tape)
{
    const int wg = S.wall_begin + wl;
    const V3<double> out = mk(walls.n[3 * wg], walls.n[3 * wg + 1], walls.n[3 * wg + 2]);
    const V3<double> org = mk(walls.o[3 * wg], walls.o[3 * wg + 1], walls.o[3 * wg + 2]);
    const double depth = rad - dot(p - org, out);
    if (depth <= 0.0) return;
    bool fresh;
    const int slot = acquire(hw, kWSlots, ci, (uint64_t)wl + 1ull, step, whw, bhigh, &fresh);
    if (slot < 0) { ++bover; return; }
    T* hv = hw.val + ((size_t)ci * kWSlots + slot) * kHV;
    if (tape.pw) {
        const int k = atomicAdd(tape.pw_count, 1);
        if (k < tape.pw_cap) {
            tape.pw[k] = make_int4(ci, wl, ci * kWSlots + slot, fresh ? 1 : 0);
            for (int a = 0; a < kHV; ++a) tape.pw_h[(size_t)k * kHV + a] = (double)hv[a];
        } else {
            atomicOr(tape.overflow, 2);
        }
    }
    const V3<double> vel = mk(c.vx[ci], c.vy[ci], c.vz[ci]);
    const V3<double> om = rot_iv(o.qw[w], o.qx[w], o.qy[w], o.qz[w], mk(o.wx[w], o.wy[w], o.wz[w]));
    const V3<double> off = c.ox ? mk(c.ox[ci], c.oy[ci], c.oz[ci]) : mk(0.0, 0.0, 0.0);
    V3<T> f, cpl;
    wall_law<T>(mat<T>(S.pw, S.pwf), T(dt_eff), cvt<T>(out), T(depth), T(rad), T(o.mass[w]), cvt<T>(vel), cvt<T>(om),
                hv, f, cpl);
    const V3<double> fd = cvt<double>(f);
    wF = wF + fd;
    wT = wT + (cvt<double>(cpl) + cross(off, fd));
}

// Planar walls (wallContact, :975-1063) in two passes.  The components'
// wall slots were expired by the sweep, which runs first; wall, particle and
// body slots are separate arrays, so the slots each acquires are those of
// the reference's order (all expiries, then walls, particles, bodies).
//
// Pass 1, per component in input order: FP32 rejection on the wall planes
// (a wall is skipped only when the particle is certainly clear of it; tol
// bounds the FP32 error of the plane distance for these coordinates).  The
// components with a wall that may touch go to a compact list with their
// candidate mask (walls past the 32nd are always candidates: a scene with
// more than 32 walls lists every component by setting bit 31, which only
// adds wall 31 to the exact test); every wall
// flag of the step starts cleared.  The list's order does not matter: pass
// 2 handles each component whole, in one thread, so the FP64 work runs in
// full warps instead of one lane in every warp that holds a wall particle.
template <typename T>
__global__ void __launch_bounds__(256) k_walls_probe(Comps c, Owners o, const SceneC* __restrict__ sc, Walls walls,
                                                     Hist<T> hw, Counters k, unsigned char* wflag, int2* wlist)
{
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned cand = 0u;
    if (ci < c.n) {
        // expireHistory (:1109-1117) of the wall slots, before pass 2
        // acquires any for this step
        expire<false>(hw, kWSlots, ci, *k.step);
        wflag[ci] = 0;
        const SceneC& S = sc[o.scene[c.owner[ci]]];
        if (S.wall_count > 0) {
            const float pfx = f32_rn(c.x[ci]), pfy = f32_rn(c.y[ci]), pfz = f32_rn(c.z[ci]), rf = f32_rn(c.radius[ci]);
            const float tol = 1e-6f + 1e-6f * (fabsf(pfx) + fabsf(pfy) + fabsf(pfz));
            const int nw32 = min(S.wall_count, 32);
            for (int wl = 0; wl < nw32; ++wl) {
                const float4 pl = walls.plane[S.wall_begin + wl];
                const float distf = fmaf(pl.x, pfx, fmaf(pl.y, pfy, pl.z * pfz)) - pl.w;
                if (distf - rf <= tol + 1e-6f * fabsf(pl.w)) cand |= 1u << wl;
            }
            if (S.wall_count > 32) cand |= 0x80000000u;
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, cand != 0u);
    if (m) {
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(k.wl_total, __popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (cand) wlist[base + __popc(m & ((1u << lane) - 1u))] = make_int2(ci, (int)cand);
    }
}

// Pass 2, one thread per listed component: the exact FP64 depth, slot
// acquisition and wall law for its candidate walls in ascending order.
template <typename T>
__global__ void __launch_bounds__(128) k_walls_law(Comps c, Owners o, const SceneC* __restrict__ sc, Walls walls,
                                                   Hist<T> hw, Contacts<T> ct, Counters k, double dt_eff)
{
    const int step = *k.step;
    const int total = *k.wl_total;
    const StepTape tape = tape_at(ct.tape);
    int bover = 0, bhigh = 0;
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < total; item += gridDim.x * blockDim.x) {
        const int2 e = ct.wlist[item];
        const int ci = e.x;
        unsigned cand = (unsigned)e.y;
        const int w = c.owner[ci];
        const SceneC& S = sc[o.scene[w]];
        const V3<double> p = mk(c.x[ci], c.y[ci], c.z[ci]);
        const double rad = c.radius[ci];
        V3<double> wF = mk(0.0, 0.0, 0.0), wT = mk(0.0, 0.0, 0.0);
        int whw = hw.hw[ci];
        for (; cand; cand &= cand - 1u)
            wall_contact<T>(c, o, S, walls, hw, ci, w, __ffs(cand) - 1, p, rad, step, dt_eff, whw, bhigh, bover, wF, wT,
                            tape);
        for (int wl = 32; wl < S.wall_count; ++wl)
            wall_contact<T>(c, o, S, walls, hw, ci, w, wl, p, rad, step, dt_eff, whw, bhigh, bover, wF, wT, tape);
        hw.hw[ci] = whw;
        const bool hit = wF.x != 0.0 || wF.y != 0.0 || wF.z != 0.0 || wT.x != 0.0 || wT.y != 0.0 || wT.z != 0.0;
        if (hit) {
            ct.wflag[ci] = 1;
            double* wr = ct.wres + 6 * (size_t)ci;
            wr[0] = wF.x; wr[1] = wF.y; wr[2] = wF.z; wr[3] = wT.x; wr[4] = wT.y; wr[5] = wT.z;
        }
    }
    block_add(k.bover, bover);
    block_max(k.bhigh, bhigh);
}

// Adjoint tape of the particle contacts of this step (FP64 form), between
// the sweep and the law: component, partner, history slot index, new flag,
// and the slot's history before the law updates it.
template <typename T>
__global__ void k_tape_pp(Recs r, Hist<T> hp, Contacts<T> ct, Counters k)
{
    const StepTape tp = tape_at(ct.tape);
    const int total = *k.ct_total;
    if (blockIdx.x == 0 && threadIdx.x == 0 && total > tp.pp_cap) atomicOr(tp.overflow, 1);
    const int n = min(total, tp.pp_cap);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int4 e = ct.ent[q];
        tp.pp[q] = make_int4(r.meta[e.x].x, r.meta[e.y].x, e.z, tp.pp_new[q]);
        const T* hv = hp.val + (size_t)e.z * kHV;
        for (int a = 0; a < kHV; ++a) tp.pp_h[(size_t)q * kHV + a] = (double)hv[a];
    }
}

// ------------------------------------------------------------- particle sweep
constexpr int kMaxContacts = kPSlots;
constexpr int kCandidates = 96;  // FP32-prefilter survivors held before the exact pass

// Residency asked of the latency-bound per-component and per-contact kernels
// (blocks per SM at their launch width; the register budget follows): the
// sweep 8 blocks of 128 (64 registers), the mixed particle law 4 of 256 (64)
// and the mixed owner sum 6 of 256 (40).  Left to itself the compiler gave
// them 96, 78 and 72 registers, and so 5, 3 and 3 blocks.  The FP64 forms
// keep the residency they had (the particle law is FP64-pipe bound).
constexpr int kSweepMinBlocks = 8;
template <typename T> constexpr int kPpLawMinBlocks = sizeof(T) == sizeof(float) ? 4 : 2;
template <typename T> constexpr int kOwnerSumMinBlocks = sizeof(T) == sizeof(float) ? 6 : 3;
constexpr int kCertain = 1 << 30;  // staged candidate flag: contact decided by the FP32 test

// Exact part of the reference's overlap test for one candidate (:587-597):
// same owner skipped, FP64 d^2 with the reference's contraction, strict
// inequality against (ri + rj)^2, coincident centres skipped.  Kept out of
// line so the FP64 work runs for prefilter survivors only.
__device__ __noinline__ bool exact_contact(const D4* __restrict__ pos, const int4* __restrict__ meta, int u, int owner,
                                           double px, double py, double pz, double pr, int& cid)
{
    const int4 mj = meta[u];
    if (mj.y == owner) return false;
    const D4 pj = pos[u];
    const V3<double> delta = mk(pj.x - px, pj.y - py, pj.z - pz);
    const double d2 = distance_squared(delta);
    const double rs = pr + pj.w;
    if (d2 >= rs * rs || d2 <= 1.0e-28) return false;
    cid = mj.z;
    return true;
}

// The sweep of one component from its neighbour list (the pairs within
// r_i + r_j + skin at the list's build, no component having moved half the
// skin since): each listed partner's cell is adjacent, and the same FP32
// test and exact FP64 test as the cell sweep decide the contact.  The
// contacts are then taken in the cell sweep's order (column (dx, dy), then
// sorted position), so the slots, the list and every sum come out as the
// cell sweep's.  Returns the contact count; stage_t / stage_s as k_sweep.
template <typename T>
__device__ int sweep_list_one(const Grid& g, const Recs& r, const SceneC* __restrict__ sc, Hist<T> hp, Counters k,
                              int t, int nvalid, int nc, int step, int* stage_t, int* stage_s, int& pover, int& phigh)
{
    const int4 meta = r.meta[t];
    const int ci = meta.x, owner = meta.y, s = meta.w;
    const int4 cell = r.cell[t];
    const D4 pi = r.pos[t];
    const float4 fi = r.relf[t];
    const float mesh_f = sc[s].mesh_f, margin_f = sc[s].margin_f;
    const float offx[3] = {-mesh_f - fi.x, -fi.x, mesh_f - fi.x};
    const float offy[3] = {-mesh_f - fi.y, -fi.y, mesh_f - fi.y};
    const float offz[3] = {-mesh_f - fi.z, -fi.z, mesh_f - fi.z};
    // the list is entry-major (entry q of component ci at q * nc + ci); its
    // first four entries load with its length
    const int* L = k.nl_idx + ci;
    const int l0 = L[0], l1 = L[nc], l2 = L[2 * (size_t)nc], l3 = L[3 * (size_t)nc];
    const int nn = min(k.nl_cnt[ci], kNL);
    expire<true>(hp, kPSlots, ci, step);
    int phw = hp.hw[ci];
    int fkey[kNL], fcid[kNL];
    int found = 0;
    for (int q = 0; q < nn; ++q) {
        const int j = q == 0 ? l0 : q == 1 ? l1 : q == 2 ? l2 : q == 3 ? l3 : L[(size_t)q * nc];
        const int u = g.pos_of[j];
        if (u < 0 || u >= nvalid) continue;
        const int4 mj = r.meta[u];
        if (mj.x != j) continue;  // not in this step's grid
        const int4 cj = r.cell[u];
        const int dx = cj.x - cell.x, dy = cj.y - cell.y, dz = cj.z - cell.z;
        if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) continue;
        const float4 fj = r.relf[u];
        const float ddx = fj.x + offx[dx + 1], ddy = fj.y + offy[dy + 1], ddz = fj.z + offz[dz + 1];
        const float rsf = fj.w + fi.w + margin_f;
        const float dd2 = ddx * ddx + ddy * ddy + ddz * ddz;
        if (dd2 >= rsf * rsf) continue;
        const float rin = rsf - 2.f * margin_f;
        int cid;
        if (dd2 < rin * rin && dd2 > 4.f * margin_f * margin_f) {
            if (mj.y == owner) continue;
            cid = mj.z;
        } else if (!exact_contact(r.pos, r.meta, u, owner, pi.x, pi.y, pi.z, pi.w, cid)) {
            continue;
        }
        // insert in the cell sweep's order: column, then sorted position
        const int key = ((dx + 1) * 3 + (dy + 1)) * (1 << 27) + u;
        int at = found++;
        while (at > 0 && fkey[at - 1] > key) {
            fkey[at] = fkey[at - 1];
            fcid[at] = fcid[at - 1];
            --at;
        }
        fkey[at] = key;
        fcid[at] = cid;
    }
    int count = 0;
    for (int q = 0; q < found; ++q) {
        if (count >= kMaxContacts) { ++pover; continue; }
        bool fresh;
        const int slot = acquire(hp, kPSlots, ci, (uint64_t)(uint32_t)fcid[q] + 1ull, step, phw, phigh, &fresh);
        if (slot < 0) { ++pover; continue; }
        stage_t[count] = fkey[q] & ((1 << 27) - 1);
        stage_s[count] = slot | (fresh ? 0x100 : 0);
        ++count;
    }
    hp.hw[ci] = phw;
    return count;
}

// Whether one of the 27 cells around sorted position t held a mover this
// step (a component past half the skin since the lists' build): such a
// component sweeps the cells instead of its list.  Every list and build
// position is from the same build, so a component with no mover in its
// cells and any partner it touches have each moved at most half the skin
// since: the pair is listed.  Cell adjacency is symmetric, so the movers
// mark the cells around theirs (k_gather_geom) and the component reads its
// own cell's mark.
__device__ __forceinline__ bool mover_near(const Recs& r, const Counters& k, int t, int step)
{
    return k.nl_hot[r.cell[t].w] == step;
}

// One thread per component in cell order: the reference's 27-cell sweep
// (:1124-1146) over the cell start table, in the reference's order (dx, dy,
// dz ascending; members of a cell in ascending component order).  For each
// (dx, dy) column the up to three z-cells are one contiguous range of the
// sorted order.  Phase 1 keeps candidates that pass an FP32 test on
// cell-relative coordinates (margin 1e-5 cell edges); phase 2 runs the exact
// FP64 test and the history slot acquisition (acquireHistorySlot, :190-215)
// on them in order.  Contacts go to a flat list; results are stored per
// (slot rank, component) so the owner sum reads them coalesced.
template <typename T>
__global__ void __launch_bounds__(128, kSweepMinBlocks) k_sweep(Grid g, Recs r, const SceneC* __restrict__ sc, Hist<T> hp,
                                               Contacts<T> ct, Counters k, int nc)
{
    const int step = *k.step;
    const int nvalid = *g.nvalid;
    // neighbour lists: this step sweeps the lists, or sweeps the cells and
    // rebuilds them (kNL partners within r_i + r_j + skin per component)
    const bool from_lists = k.nl_on && *k.nl_flag == 0;
    const bool build = k.nl_on && !from_lists;
    const bool movers = from_lists && k.nl_flag[3] > 0;  // any cell stamped this step
    int pover = 0, phigh = 0, found = 0;
    // grid-stride over blocks of sorted positions: the launch may use fewer
    // blocks than positions so that the kernels beside it find free slots
    for (int t0 = blockIdx.x * blockDim.x; t0 < nvalid; t0 += gridDim.x * blockDim.x) {
    const int t = t0 + threadIdx.x;
    int count = 0;
    int stage_t[kCandidates];
    int stage_s[kMaxContacts];
    int ci = -1;
    if (t < nvalid && from_lists && !(movers && mover_near(r, k, t, step))) {
        ci = r.meta[t].x;
        count = sweep_list_one(g, r, sc, hp, k, t, nvalid, nc, step, stage_t, stage_s, pover, phigh);
        ct.cnt[ci] = count;
    } else if (t < nvalid) {
        const int4 meta = r.meta[t];
        ci = meta.x;
        const int owner = meta.y, s = meta.w;
        const int4 cell = r.cell[t];
        const D4 pi = r.pos[t];
        const int* lay = g.scene_layout + 8 * s;
        const float4 fi = r.relf[t];
        const float mesh_f = sc[s].mesh_f, margin_f = sc[s].margin_f;
        const float offx[3] = {-mesh_f - fi.x, -fi.x, mesh_f - fi.x};
        const float offy[3] = {-mesh_f - fi.y, -fi.y, mesh_f - fi.y};
        const float offz[3] = {-mesh_f - fi.z, -fi.z, mesh_f - fi.z};
        const int z0 = max(cell.z - 1, lay[2]), z1 = min(cell.z + 1, lay[2] + lay[5] - 1);
        const float skin_f = sc[s].skin_f;
        int* nl = build ? k.nl_idx + ci : nullptr;  // entry-major: entry q at nl[q * nc]
        int nlist = 0;
        // expireHistory (:1109-1117) for the component's particle slots,
        // before any slot of this step is acquired (the wall and body slots
        // expire in their own probes)
        expire<true>(hp, kPSlots, ci, step);
        int phw = hp.hw[ci];
        int pending = 0;  // candidates in stage_t[count .. count + pending)
        // Phase 2 over the staged candidates, in order.  A candidate staged
        // with kCertain passed the FP32 test with the rounding margin to
        // spare on both sides (d < r_i + r_j and d > 0 hold in FP64 too), so
        // only the owner check and its key need the record.
        auto exact_pass = [&]() {
            const int first = count, last = count + pending;
            for (int q = first; q < last; ++q) {
                const int su = stage_t[q];
                const int u = su & ~kCertain;
                int cid;
                if (su & kCertain) {
                    const int4 mj = r.meta[u];
                    if (mj.y == owner) continue;
                    cid = mj.z;
                } else if (!exact_contact(r.pos, r.meta, u, owner, pi.x, pi.y, pi.z, pi.w, cid)) {
                    continue;
                }
                if (count >= kMaxContacts) { ++pover; continue; }
                bool fresh;
                const int slot = acquire(hp, kPSlots, ci, (uint64_t)(uint32_t)cid + 1ull, step, phw, phigh, &fresh);
                if (slot < 0) { ++pover; continue; }
                stage_t[count] = u;
                stage_s[count] = slot | (fresh ? 0x100 : 0);
                ++count;
            }
            pending = 0;
        };
        for (int dx = -1; dx <= 1; ++dx) {
            const int nx = cell.x + dx;
            if (nx < lay[0] || nx >= lay[0] + lay[3]) continue;
            const float ox = offx[dx + 1];
            for (int dy = -1; dy <= 1; ++dy) {
                const int ny = cell.y + dy;
                if (ny < lay[1] || ny >= lay[1] + lay[4]) continue;
                const float oy = offy[dy + 1];
                const int row = lay[6] + ((nx - lay[0]) * lay[4] + (ny - lay[1])) * lay[5] - lay[2];
                // the z-cells z0..z1 of this column are one contiguous range
                // [b0, e) of the sorted order, split at b1 and b2
                const int b0 = g.cell_start[row + z0];
                const int e = g.cell_start[row + z1 + 1];
                const int b1 = z1 >= z0 + 1 ? g.cell_start[row + z0 + 1] : e;
                const int b2 = z1 >= z0 + 2 ? g.cell_start[row + z0 + 2] : e;
                const float oz0 = offz[z0 - cell.z + 1];
                const float oz1 = z1 >= z0 + 1 ? offz[z0 - cell.z + 2] : 0.f;
                const float oz2 = z1 >= z0 + 2 ? offz[z0 - cell.z + 3] : 0.f;
                // four candidates per iteration: their loads are issued
                // together, the survivors are appended in order
                for (int u0 = b0; u0 < e; u0 += 4) {
                    float4 fj[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        fj[q] = (u0 + q < e) ? r.relf[u0 + q] : make_float4(1e30f, 1e30f, 1e30f, 0.f);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int u = u0 + q;
                        const float oz = u < b1 ? oz0 : (u < b2 ? oz1 : oz2);
                        const float ddx = fj[q].x + ox, ddy = fj[q].y + oy, ddz = fj[q].z + oz;
                        const float rsf = fj[q].w + fi.w + margin_f;
                        const float dd2 = ddx * ddx + ddy * ddy + ddz * ddz;
                        if (build && u != t) {
                            const float rsb = rsf + skin_f;
                            if (dd2 < rsb * rsb) {
                                if (nlist < kNL) nl[(size_t)nlist * nc] = r.meta[u].x;
                                ++nlist;
                            }
                        }
                        if (dd2 >= rsf * rsf) continue;
                        const float rin = rsf - 2.f * margin_f;
                        const bool certain = dd2 < rin * rin && dd2 > 4.f * margin_f * margin_f;
                        if (count + pending == kCandidates) exact_pass();
                        stage_t[count + pending] = certain ? (u | kCertain) : u;
                        ++pending;
                    }
                }
            }
        }
        exact_pass();
        hp.hw[ci] = phw;
        ct.cnt[ci] = count;
        if (build) {
            k.nl_cnt[ci] = min(nlist, kNL);
            if (nlist > kNL) k.nl_flag[1] = 1;
            double* xr = k.nl_xref + 3 * (size_t)ci;
            xr[0] = pi.x; xr[1] = pi.y; xr[2] = pi.z;
        }
    }
    // the warp's contacts take one range of the flat list (no block barrier:
    // a warp that finishes its candidates early goes on to its next pass)
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int incl = count;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    const int wtotal = __shfl_sync(FULL, incl, 31);
    int wbase = 0;
    if (lane == 31 && wtotal) wbase = atomicAdd(k.ct_total, wtotal);
    const int base = __shfl_sync(FULL, wbase, 31) + incl - count;
    for (int q = 0; q < count; ++q) {
        ct.ent[base + q] = make_int4(t, stage_t[q], ci * kPSlots + (stage_s[q] & 0xff), q * nc + ci);
        if (ct.tape.pp_new) ct.tape.pp_new[base + q] = (unsigned char)(stage_s[q] >> 8);
    }
    found += count;
    }
    block_add(k.pcontacts, found);
    block_add(k.pover, pover);
    block_max(k.phigh, phigh);
}

// ------------------------------------------------------------------ PP law
// particleContact (:579-706) for one contact of the flat list.  Everything
// the law reads is loaded before any arithmetic (records through the
// read-only path, the history slot as vectors), so the loads of a contact
// are in flight together.
template <typename T>
__global__ void __launch_bounds__(256, kPpLawMinBlocks<T>) k_pp_law(Recs r, const SceneC* __restrict__ sc, Hist<T> hp, Contacts<T> ct,
                                                Counters k, double dt_eff, int nscenes)
{
    const int total = *k.ct_total;
    const T dtT = T(dt_eff);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        const int4 e = __ldg(&ct.ent[q]);
        const D4 pi = ldg_d4(&r.pos[e.x]), pj = ldg_d4(&r.pos[e.y]);
        const int s = nscenes > 1 ? __ldg(&r.meta[e.x].w) : 0;
        T h[9];
        T* hv = hp.val + (size_t)e.z * kHV;
        hv_load(hv, h);
        V3<T> erv, mrv, ewi, ewj, mwi, mwj;
        T mi_, mj_;
        if constexpr (sizeof(T) == sizeof(double)) {
            const D4 vi = ldg_d4(&r.v[e.x]), vj = ldg_d4(&r.v[e.y]);
            const D4 ui = ldg_d4(&r.vm[e.x]), uj = ldg_d4(&r.vm[e.y]);
            const D4 wi = ldg_d4(&r.w[e.x]), wj = ldg_d4(&r.w[e.y]);
            const D4 xi = ldg_d4(&r.wm[e.x]), xj = ldg_d4(&r.wm[e.y]);
            erv = d3(vj) - d3(vi);
            mrv = d3(uj) - d3(ui);
            ewi = d3(wi); ewj = d3(wj);
            mwi = d3(xi); mwj = d3(xj);
            mi_ = vi.w; mj_ = vj.w;
        } else {
            const float4 vi = __ldg(&r.vf[e.x]), vj = __ldg(&r.vf[e.y]);
            const float4 ui = __ldg(&r.vmf[e.x]), uj = __ldg(&r.vmf[e.y]);
            const float4 wi = __ldg(&r.wf[e.x]), wj = __ldg(&r.wf[e.y]);
            const float4 xi = __ldg(&r.wmf[e.x]), xj = __ldg(&r.wmf[e.y]);
            erv = f3(vj) - f3(vi);
            mrv = f3(uj) - f3(ui);
            ewi = f3(wi); ewj = f3(wj);
            mwi = f3(xi); mwj = f3(xj);
            mi_ = vi.w; mj_ = vj.w;
        }
        const V3<double> delta = mk(pj.x - pi.x, pj.y - pi.y, pj.z - pi.z);
        const double d2 = distance_squared(delta);
        const double rs = pi.w + pj.w;
        T d, depth;
        V3<T> n;
        if constexpr (sizeof(T) == sizeof(double)) {
            const double dd = sqrt(d2);
            d = dd;
            depth = rs - dd;
            n = delta * (1.0 / dd);
        } else {
            // Overlap from the FP64 difference of squares, the rest in FP32.
            const double num = __fma_rn(rs, rs, -d2);
            const float df = sqrtf(f32_rn(d2));
            d = df;
            depth = f32_rn(num) / (f32_rn(rs) + df);
            n = cvt<float>(delta) * (1.0f / df);
        }
        const SceneC& S = sc[s];
        V3<T> f, cpl;
        pp_law<T>(mat<T>(S.pp, S.ppf), dtT, n, d, depth, cv<T>(d2), cv<T>(pi.w), cv<T>(pj.w), mi_, mj_, erv, mrv, ewi,
                  ewj, mwi, mwj, h, f, cpl);
        hv_store(hv, h);
        if (r.off) cpl = cpl + cross(cvt<T>(d3(r.off[e.x])), f);
        T* out = ct.res + 6 * (size_t)e.w;
        if constexpr (sizeof(T) == sizeof(double)) {
            double2* o2 = reinterpret_cast<double2*>(out);
            o2[0] = make_double2(f.x, f.y); o2[1] = make_double2(f.z, cpl.x); o2[2] = make_double2(cpl.y, cpl.z);
        } else {
            float2* o2 = reinterpret_cast<float2*>(out);
            o2[0] = make_float2(f.x, f.y); o2[1] = make_float2(f.z, cpl.x); o2[2] = make_float2(cpl.y, cpl.z);
        }
    }
}


// ------------------------------------------------------------------- PT

__device__ __noinline__ double circle_triangle_area_fp64(V3<double> n, V3<double> ra, V3<double> rb, V3<double> rc,
                                                        double r)
{
    return circle_triangle_area<double>(n, ra, rb, rc, r);
}

// bodyTriangleAreaScale (:380-407); also returns distance along the outward
// normal.
template <typename T>
__device__ double tri_area_scale(const double* W, V3<double> p, double r, double& dist)
{
    if constexpr (sizeof(T) == sizeof(double)) return tri_area_scale64(W, p, r, dist);
    const V3<double> n = mk(W[12], W[13], W[14]);
    const V3<double> a = mk(W[3], W[4], W[5]);
    dist = dot(n, p - a);
    if (dist <= 0.0) return 0.0;
    const double c2 = r * r - dist * dist;
    if (c2 <= 1.0e-30) return 0.0;
    const V3<double> ce = p - n * dist;
    const V3<double> ra = a - ce, rb = mk(W[6], W[7], W[8]) - ce, rc = mk(W[9], W[10], W[11]) - ce;
    // Disk and triangle disjoint (disk centre farther from the triangle's
    // centroid than the disk radius plus the triangle's circumradius about
    // it, W[15]): the reference's edge sum then cancels to rounding noise,
    // far below its 1e-12 threshold, so the scale is 0 either way.
    {
        const V3<double> cen = (ra + rb + rc) * (1.0 / 3.0);
        const double reach = (sqrt(c2) + W[15]) * (1.0 + 1e-9);
        if (dot(cen, cen) > reach * reach) return 0.0;
    }
    double area;
    if constexpr (sizeof(T) == sizeof(double)) {
        area = circle_triangle_area<double>(n, ra, rb, rc, sqrt(c2));
    } else {
        // FP32 area, except where it decides the threshold: a scale below
        // 1e-4 (a disk that grazes the triangle, where FP32 cancellation
        // noise exceeds the 1e-12 cut) is recomputed in FP64, so the set of
        // manifolds is the FP64 one
        area = f64_of(circle_triangle_area<float>(cvt<float>(n), cvt<float>(ra), cvt<float>(rb), cvt<float>(rc),
                                                  sqrtf(f32_rn(c2))));
        if (!(area >= 1.0e-4 * kPi * c2)) area = circle_triangle_area_fp64(n, ra, rb, rc, sqrt(c2));
    }
    if (area <= 0.0) return 0.0;
    const double sc = fmin(1.0, area / (kPi * c2));
    return sc > 1.0e-12 ? sc : 0.0;
}

// Conservative FP32 rejection of a particle-triangle pair: false only when
// tri_area_scale is certainly 0 (the particle is not strictly above the
// triangle's plane within its radius, or the contact disk cannot reach the
// triangle).  tol bounds the FP32 error of the plane distance; it scales
// with the coordinates' magnitude.
struct PtProbe {
    float px, py, pz, r, tol;
};
__device__ __forceinline__ PtProbe pt_probe(V3<double> p, double r)
{
    PtProbe q;
    q.px = f32_rn(p.x); q.py = f32_rn(p.y); q.pz = f32_rn(p.z); q.r = f32_rn(r);
    q.tol = 1e-6f + 1e-6f * (fabsf(q.px) + fabsf(q.py) + fabsf(q.pz));
    return q;
}
__device__ __forceinline__ bool pt_may_touch(const float4* __restrict__ tf, int tri, const PtProbe& q)
{
    const float4 A = __ldg(&tf[2 * (size_t)tri]);
    const float tol = q.tol + 1e-6f * fabsf(A.w);
    const float dist = fmaf(A.x, q.px, fmaf(A.y, q.py, A.z * q.pz)) - A.w;
    if (dist <= -tol || dist >= q.r + tol) return false;
    const float4 B = __ldg(&tf[2 * (size_t)tri + 1]);
    const float dlo = fmaxf(dist - tol, 0.f);
    const float reach = sqrtf(fmaxf(q.r * q.r - dlo * dlo, 0.f)) + B.w + 4.f * tol;
    const float cx = B.x - (q.px - A.x * dist), cy = B.y - (q.py - A.y * dist), cz = B.z - (q.pz - A.z * dist);
    return cx * cx + cy * cy + cz * cz <= reach * reach;
}

// Per sorted position: can any triangle of its cell give a nonzero area
// scale (the condition of a manifold, :1154-1183)?  FP32 rejection only: a
// position may be kept without a manifold (the law kernel then finds none),
// never dropped with one.  Triangle loads go four at a time.
__device__ __forceinline__ bool pt_cell_may_touch(const Tris& tris, int tb, int te, const PtProbe& q)
{
    for (int e0 = tb; e0 < te; e0 += 4) {
        int tri[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) tri[u] = e0 + u < te ? __ldg(&tris.ttri[e0 + u]) : -1;
        bool hit = false;
#pragma unroll
        for (int u = 0; u < 4; ++u) hit |= tri[u] >= 0 && pt_may_touch(tris.tf, tri[u], q);
        if (hit) return true;
    }
    return false;
}

// The contact items of a step in one launch: per sorted position, the expiry
// of its body slots (expireHistory, :1109-1117, before the law kernels
// acquire any) and the probe; then its rank among the kept positions (block
// scan plus the tiles before it, by single-pass look-back, ScanState) gives
// the item list in sorted order and each component's item index (-1: none).
template <typename TB, int kPtTile>
__global__ void __launch_bounds__(kPtTile) k_pt_items(Grid g, Recs r, Tris tris, Hist<TB> hb, Counters k, int* clist,
                                                      int* pt_index, int* ctotal, ScanState st, unsigned* err)
{
    __shared__ int s_tile, s_prefix;
    const int nvalid = *g.nvalid;
    const int step = *k.step;
    const int ntiles = min((nvalid + kPtTile - 1) / kPtTile, st.max_tiles);
    const unsigned epoch = st.ctl[2];
    if (nvalid == 0 && blockIdx.x == 0 && threadIdx.x == 0) *ctotal = 0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(st.ctl, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= ntiles) break;
        const int t = tile * kPtTile + threadIdx.x;
        int hit = 0, ci = -1;
        if (t < nvalid) {
            ci = g.sorted_id[t];
            expire<false>(hb, kBSlots, ci, step);
            const int lin = r.cell[t].w;
            const int tb = tris.tcell_start[lin];
            const int te = min(tris.tcell_start[lin + 1], tris.capacity);
            if (te > tb) {
                const D4 p4 = r.pos[t];
                hit = pt_cell_may_touch(tris, tb, te, pt_probe(d3(p4), p4.w)) ? 1 : 0;
            }
        }
        int total;
        const int ex = block_exclusive_scan_c(hit, total);
        if (threadIdx.x == 0) scan_publish(st, tile, total, epoch, tile == 0 ? 2u : 1u);
        if (threadIdx.x < 32) {
            const int prefix = tile == 0 ? 0 : scan_lookback(st, tile, epoch, err);
            if (threadIdx.x == 0) {
                if (tile > 0) scan_publish(st, tile, prefix + total, epoch, 2u);
                s_prefix = prefix;
            }
        }
        __syncthreads();
        if (t < nvalid) {
            if (hit) {
                clist[s_prefix + ex] = t;
                pt_index[ci] = s_prefix + ex;
            } else {
                pt_index[ci] = -1;
            }
        }
        if (tile == ntiles - 1 && threadIdx.x == 0) *ctotal = s_prefix + total;
        __syncthreads();  // s_tile, s_prefix are reused by the next tile
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(st.ctl + 1, 1u) == gridDim.x - 1) {
            st.ctl[0] = 0u;
            st.ctl[1] = 0u;
            atomicAdd(st.ctl + 2, 1u);
        }
    }
}

// ---------------------------------------------------------- PT laws
// The particle-side inputs of one contact item and the body-side inputs of
// one body, and the three pieces of the reference's body contact that both
// PT kernels below share.
struct PtItem {
    V3<double> p, ev, mv, ew, mw, off;
    double rad, mass;
};
struct PtBody {
    V3<double> center, wb, bv;
    const double* bq;
};

__device__ __forceinline__ PtItem pt_item(const Comps& c, const Owners& o, const Recs& r, int t, int ci, int w,
                                          double dt_eff)
{
    PtItem it;
    const D4 p4 = r.pos[t];
    it.p = d3(p4);
    it.rad = p4.w;
    it.mass = o.mass[w];
    // FP64 velocities straight from the state (the mixed form keeps FP32
    // rows only for the particle-particle law).
    const bool mid = dt_eff > 0.0 && o.status[w] != -1;
    it.ev = mk(c.vx[ci], c.vy[ci], c.vz[ci]);
    it.mv = mid ? mk(c.vhx[ci], c.vhy[ci], c.vhz[ci]) : it.ev;
    const double oqw = o.qw[w], oqx = o.qx[w], oqy = o.qy[w], oqz = o.qz[w];
    it.ew = rot_iv(oqw, oqx, oqy, oqz, mk(o.wx[w], o.wy[w], o.wz[w]));
    it.mw = mid ? rot_iv(oqw, oqx, oqy, oqz, mk(o.whx[w], o.why[w], o.whz[w])) : it.ew;
    it.off = r.off ? d3(r.off[t]) : mk(0.0, 0.0, 0.0);
    return it;
}

__device__ __forceinline__ PtBody pt_body(const Bodies& bodies, int b)
{
    PtBody bd;
    bd.center = mk(bodies.c[3 * b], bodies.c[3 * b + 1], bodies.c[3 * b + 2]);
    bd.bq = bodies.q + 4 * b;
    bd.wb = rot_iv(bd.bq[0], bd.bq[1], bd.bq[2], bd.bq[3], mk(bodies.w[3 * b], bodies.w[3 * b + 1], bodies.w[3 * b + 2]));
    bd.bv = mk(bodies.v[3 * b], bodies.v[3 * b + 1], bodies.v[3 * b + 2]);
    return bd;
}

// advanceBodyManifoldHistory (:855-949): the manifold (normal mn, centre mc,
// distance md) updates the history h in place.
template <typename T>
__device__ void pt_manifold_history(const MatC& m, const PtItem& it, const PtBody& bd, V3<double> mn, V3<double> mc,
                                    double md, double dt_eff, T* h, bool& slide, bool& twist)
{
    const V3<double> arm = mc - bd.center;
    const V3<double> bvel = bd.bv + cross(bd.wb, arm);
    const V3<T> erv = cvt<T>(bvel - it.ev), mrv = cvt<T>(bvel - it.mv);
    const V3<T> n = cvt<T>(mn);
    const LawC<T> c = law_constants<T>(m, T(it.mass), T(it.rad));
    const T depth = T(it.rad - md);
    V3<T> fn = n * (-c.kN * depth) + n * (c.cN * dot(erv, n));
    fn = fn + n * (T(m.coh) * T(4.0) * c.brs);
    V3<T> tv = mrv - n * dot(mrv, n);
    tv = tv + cross(n, cvt<T>(it.mw)) * T(md);
    V3<T> st;
    limited_rates<T>(tv, tv, c.kS, c.cS, T(dt_eff), transport_tangent(hload(h, 1), n), T(m.mu) * norm(fn), st, slide);
    hstore(h, 1, st);
    const V3<T> rw = cvt<T>(bd.wb - it.mw);
    const V3<T> twr = n * dot(rw, n);
    const V3<T> rlr = (rw - twr) + cross(n, tv) * (T(0.5) / fmax(T(md), T(1.0e-14)));
    const T ms = T(m.beta) * T(it.rad) * norm(fn);
    limited_rates<T>(twr, twr, c.kT, c.cT, T(dt_eff), transport_axial(hload(h, 2), n), T(m.mu) * T(m.muT) * ms, st,
                     twist);
    hstore(h, 2, st);
    bool dummy;
    limited_rates<T>(rlr, rlr, c.kR, c.cR, T(dt_eff), transport_tangent(hload(h, 0), n), T(m.muR) * ms, st, dummy);
    hstore(h, 0, st);
}

// bodyContact (:708-853) for one triangle with read-only history: the
// particle load pf/ptq, the body-side force rf and torque bt, and the six
// body-side terms for the optional detail output.
struct PtTri {
    V3<double> pf, ptq, rf, bt, v[6];
};
template <typename T>
__device__ void pt_triangle_load(const MatC& m, const LawC<T>& c, const PtItem& it, const PtBody& bd, const double* W,
                                 double as, double dist, V3<T> hroll, V3<T> htan, V3<T> htw, PtTri& o)
{
    const double depthd = it.rad - dist;
    const V3<double> nout = mk(W[12], W[13], W[14]);
    const V3<double> ce = it.p - nout * dist;
    const V3<double> arm = ce - bd.center;
    const V3<double> bvel = bd.bv + cross(bd.wb, arm);
    const V3<T> n = cvt<T>(nout * -1.0);
    const V3<T> rv = cvt<T>(bvel - it.ev);
    const V3<T> wp = cvt<T>(it.ew);
    const T depth = T(depthd), distT = T(dist);
    V3<T> fn = n * (-c.kN * depth) + n * (c.cN * dot(rv, n));
    fn = fn + n * (T(m.coh) * T(4.0) * c.brs);
    V3<T> tv = rv - n * dot(rv, n);
    tv = tv + cross(n, wp) * distT;
    V3<T> st;
    bool y;
    const V3<T> fr = limited_rates<T>(tv, tv, c.kS, c.cS, T(0), transport_tangent(htan, n), T(m.mu) * norm(fn), st, y);
    const V3<T> rw = cvt<T>(bd.wb) - wp;
    const V3<T> twr = n * dot(rw, n);
    const V3<T> rlr = (rw - twr) + cross(n, tv) * (T(0.5) / fmax(distT, T(1.0e-14)));
    const T ms = T(m.beta) * T(it.rad) * norm(fn);
    const V3<T> tw = limited_rates<T>(twr, twr, c.kT, c.cT, T(0), transport_axial(htw, n), T(m.mu) * T(m.muT) * ms,
                                      st, y);
    const V3<T> rl = limited_rates<T>(rlr, rlr, c.kR, c.cR, T(0), transport_tangent(hroll, n), T(m.muR) * ms, st, y);
    const V3<double> fnd = cvt<double>(fn), frd = cvt<double>(fr);
    o.pf = (fnd + frd) * as;
    const V3<double> nd = cvt<double>(n);
    const V3<double> cm = cvt<double>(tw) + cvt<double>(rl);
    const V3<double> cpl = (cm + cross(nd, frd) * dist) * as;
    o.ptq = cpl + cross(it.off, o.pf);
    const V3<double> bnf = fnd * (-as), bfr = frd * (-as);
    const V3<double> bnt = cross(arm, fnd) * (-as), bft = cross(arm, frd) * (-as);
    const V3<double> btw = cvt<double>(tw) * (-as), brl = cvt<double>(rl) * (-as);
    o.bt = (bnt + bft) + (btw + brl);
    o.rf = mk(bnf.x + bfr.x, bnf.y + bfr.y, bnf.z + bfr.z);
    o.v[0] = bnf; o.v[1] = bfr; o.v[2] = bnt; o.v[3] = bft; o.v[4] = btw; o.v[5] = brl;
}

// observeBodyMicrostateKernel (:1226-1356) for one manifold, fused; th and
// twh are the updated tangent and twist history.
__device__ void pt_microstate(const MatC& m, const PtItem& it, const PtBody& bd, V3<double> mn, V3<double> mc,
                              double md, double tot, V3<double> th, V3<double> twh, double* mcr)
{
    const double rad = it.rad;
    const V3<double> arm = mc - bd.center;
    const V3<double> bvel = bd.bv + cross(bd.wb, arm);
    const V3<double> rv = bvel - it.ev;
    const double cN = -2.0 * m.logN * sqrt(m.kN * it.mass / m.denN);
    const double brs = m.beta * rad * m.beta * rad;
    const double depth = rad - md;
    V3<double> fn = mn * (-m.kN * depth) + mn * (cN * dot(rv, mn));
    fn = fn + mn * (m.coh * 4.0 * brs);
    const double fnn = norm(fn);
    const double ms = m.beta * rad * fnn;
    const double tl = m.mu * fnn;
    const double twl = m.mu * m.muT * ms;
    const V3<double> az = rot_iv(bd.bq[0], bd.bq[1], bd.bq[2], bd.bq[3], mk(0.0, 0.0, 1.0));
    const V3<double> radial = arm - az * dot(arm, az);
    const double tu = tl > 1.0e-30 ? fmin(1.0, norm(th) / tl) : 0.0;
    const double twu = twl > 1.0e-30 ? fmin(1.0, norm(twh) / twl) : 0.0;
    const V3<double> btw = twh * (-tot), bnl = fn * (-tot), bth = th * (-tot);
    const V3<double> btt = cross(arm, bth);
    mcr[0] = fnn * tot; mcr[1] = fnn * rad * tot; mcr[2] = fnn * norm(radial) * tot;
    mcr[3] = btw.x; mcr[4] = btw.y; mcr[5] = btw.z;
    mcr[6] = norm(twh) * tot; mcr[7] = twl * tot; mcr[8] = norm(th) * tot; mcr[9] = tl * tot;
    mcr[10] = twu * tot; mcr[11] = tu * tot; mcr[12] = tot;
    mcr[13] = bnl.x; mcr[14] = bnl.y; mcr[15] = bnl.z;
    mcr[16] = bth.x; mcr[17] = bth.y; mcr[18] = bth.z;
    mcr[19] = btt.x; mcr[20] = btt.y; mcr[21] = btt.z;
}

// Contact items at or below Counters::pt_warp_items run one warp per item
// (latency bound: few items, many triangles each); above it one thread per
// item (FP64 throughput bound).  Both kernels are launched; the count on the
// device picks the one that works.

// Adjoint tape of one particle-body manifold (FP64 form): the component,
// body, history slot, whether the slot is new, the history before the
// update and the triangles with an area share, in triangle order.
template <typename T>
__device__ void tape_pb(const StepTape& tp, int ci, int b, int slot, bool fresh, const T* h, const int* tri, int ntri,
                        bool spill)
{
    const int k = atomicAdd(tp.pb_count, 1);
    if (spill || ntri > kPbTris) {
        atomicOr(tp.overflow, 8);  // more triangles with an area share than a manifold keeps
        return;
    }
    if (k >= tp.pb_cap) {
        atomicOr(tp.overflow, 4);
        return;
    }
    tp.pb[k] = make_int4(ci, b, ci * kBSlots + slot, fresh ? 1 : 0);
    int* tl = tp.pb_tri + (size_t)k * kPbTri;
    tl[0] = ntri;
    for (int q = 0; q < ntri; ++q) tl[1 + q] = tri[q];
    for (int a = 0; a < 9; ++a) tp.pb_h[(size_t)k * kHV + a] = (double)h[a];
}

// One triangle's share added to a manifold's sums (:1154-1183), as the
// warp-per-item kernel adds it.
__device__ __noinline__ void manifold_add(double& tot, V3<double>& wn, V3<double>& wc, double& wd, V3<double> p,
                                          V3<double> out, double as, double dist)
{
    const V3<double> ce = p - out * dist;
    tot += as;
    wn = wn + out * (-as);
    wc = wc + ce * as;
    wd += dist * as;
}

// ---------------------------------------------------- PT, thread per item
// The thread-per-item kernel calls the law's pieces through these wrappers,
// compiled once each (not inlined): its own code around them then cannot
// change how they round, and they give the bits that the warp-per-item
// kernel gets from the same pieces inlined (tests/test_gpu_pt_paths.py).
template <typename T>
__device__ __noinline__ double tri_area_scale_n(const double* W, V3<double> p, double r, double& dist)
{
    return tri_area_scale<T>(W, p, r, dist);
}
__device__ __noinline__ bool tri_disk_n(const double* W, V3<double> p, double r)
{
    TriDisk d;
    return tri_disk(W, p, r, d);
}
__device__ __noinline__ PtItem pt_item_n(const Comps& c, const Owners& o, const Recs& r, int t, int ci, int w,
                                         double dt_eff)
{
    return pt_item(c, o, r, t, ci, w, dt_eff);
}
__device__ __noinline__ PtBody pt_body_n(const Bodies& bodies, int b) { return pt_body(bodies, b); }
__device__ __noinline__ void pt_manifold_frame_n(double tot, V3<double> wn, V3<double> wc, double wd, V3<double>& mn,
                                                 V3<double>& mc, double& md)
{
    mn = normalized(wn);
    mc = wc * (1.0 / tot);
    md = wd / tot;
}
template <typename T>
__device__ __noinline__ void pt_manifold_history_n(const MatC& m, const PtItem& it, const PtBody& bd, V3<double> mn,
                                                   V3<double> mc, double md, double dt_eff, T* h, bool& slide,
                                                   bool& twist)
{
    pt_manifold_history<T>(m, it, bd, mn, mc, md, dt_eff, h, slide, twist);
}
template <typename T>
__device__ __noinline__ void pt_triangle_load_n(const MatC& m, const PtItem& it, const PtBody& bd, const double* W,
                                                double as, double dist, V3<T> hroll, V3<T> htan, V3<T> htw, PtTri& o)
{
    const LawC<T> lc = law_constants<T>(m, T(it.mass), T(it.rad));
    pt_triangle_load<T>(m, lc, it, bd, W, as, dist, hroll, htan, htw, o);
}
__device__ __noinline__ void pt_microstate_n(const MatC& m, const PtItem& it, const PtBody& bd, V3<double> mn,
                                             V3<double> mc, double md, double tot, V3<double> th, V3<double> twh,
                                             double* mcr)
{
    pt_microstate(m, it, bd, mn, mc, md, tot, th, twh, mcr);
}

constexpr int kTriCache = 24;

template <typename TC, typename T>
__global__ void __launch_bounds__(128) k_pt_thread(Comps c, Owners o, Recs r, const SceneC* __restrict__ sc, Tris tris,
                                                   Bodies bodies, Hist<T> hb, Contacts<TC> ct, Counters k,
                                                   double dt_eff)
{
    const int step = *k.step;
    const int total = *ct.pt_ctotal_ptr;
    if (total <= k.pt_warp_items) return;
    const StepTape tape = tape_at(ct.tape);
    int bover = 0, bhigh = 0;
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < total; item += gridDim.x * blockDim.x) {
        const int t = ct.pt_clist[item];
        const int4 meta = r.meta[t];
        const int ci = meta.x;
        const SceneC& S = sc[meta.w];
        const PtItem it = pt_item_n(c, o, r, t, ci, meta.y, dt_eff);
        const int lin = r.cell[t].w;
        const int tb = tris.tcell_start[lin];
        const int te = min(tris.tcell_start[lin + 1], tris.capacity);
        V3<double> bF = mk(0.0, 0.0, 0.0), bT = mk(0.0, 0.0, 0.0);
        int bhw = hb.hw[ci];
        const PtProbe pq = pt_probe(it.p, it.rad);
        for (int j = 0; j < S.body_count; ++j) {
            const int b = S.body_begin + j;
            double* rec = ct.pt_body + ((size_t)item * ct.nbs + j) * kPtRecord;
            for (int f = 0; f < kPtRecord; ++f) rec[f] = 0.0;
            double* outd = ct.pt_out ? ct.pt_out + ((size_t)item * ct.nbs + j) * 25 : nullptr;
            if (outd) for (int f = 0; f < 25; ++f) outd[f] = 0.0;
            // manifold sums over the component's own cell (:1154-1183); the
            // triangles with a share keep their area scale and distance
            int ctri[kTriCache];
            double cas[kTriCache], cdist[kTriCache];
            int ncache = 0;
            bool spill = false;
            double tot = 0.0, wd = 0.0;
            V3<double> wn = mk(0.0, 0.0, 0.0), wc = mk(0.0, 0.0, 0.0);
            auto add = [&](int tri, const double* W, double as, double dist) {
                manifold_add(tot, wn, wc, wd, it.p, mk(W[12], W[13], W[14]), as, dist);
                if (ncache < kTriCache) { ctri[ncache] = tri; cas[ncache] = as; cdist[ncache] = dist; ++ncache; }
                else spill = true;
            };
            // Three passes, each in triangle order, so that the lanes of a
            // warp meet in the FP64 work instead of reaching it at different
            // entries of their cells: the FP32 test over the cell's entries,
            // the FP64 tests that need no edge sum, then the areas of the
            // triangles left (one or two per item).
            int cand[kTriCache];
            int ncand = 0;
            bool many = false;
            for (int e = tb; e < te; ++e) {
                const int tri = tris.ttri[e];
                if (tris.body[tri] != b || !pt_may_touch(tris.tf, tri, pq)) continue;
                if (ncand < kTriCache) cand[ncand++] = tri;
                else many = true;
            }
            if (!many) {
                int nkeep = 0;
                for (int q = 0; q < ncand; ++q)
                    if (tri_disk_n(tris.world + 16 * (size_t)cand[q], it.p, it.rad)) cand[nkeep++] = cand[q];
                for (int q = 0; q < nkeep; ++q) {
                    const double* W = tris.world + 16 * (size_t)cand[q];
                    double dist;
                    const double as = tri_area_scale_n<T>(W, it.p, it.rad, dist);
                    if (as > 0.0) add(cand[q], W, as, dist);
                }
            } else {
                for (int e = tb; e < te; ++e) {
                    const int tri = tris.ttri[e];
                    if (tris.body[tri] != b || !pt_may_touch(tris.tf, tri, pq)) continue;
                    const double* W = tris.world + 16 * (size_t)tri;
                    double dist;
                    const double as = tri_area_scale_n<T>(W, it.p, it.rad, dist);
                    if (as > 0.0) add(tri, W, as, dist);
                }
            }
            if (tot <= 0.0) continue;
            V3<double> mn, mc;
            double md;
            pt_manifold_frame_n(tot, wn, wc, wd, mn, mc, md);
            bool fresh = false;
            const int slot = acquire(hb, kBSlots, ci, (uint64_t)(j + 1), step, bhw, bhigh, &fresh);
            if (slot < 0) { ++bover; continue; }
            T* hv = hb.val + ((size_t)ci * kBSlots + slot) * kHV;
            T h[9];
            hv_load(hv, h);
            if (tape.pb) tape_pb(tape, ci, b, slot, fresh, h, ctri, ncache, spill);
            const PtBody bd = pt_body_n(bodies, b);
            const MatC& m = S.pt;
            bool slide = false, twist = false;
            pt_manifold_history_n<T>(m, it, bd, mn, mc, md, dt_eff, h, slide, twist);
            hv_store(hv, h);
            rec[9] = (double)(1 | (slide ? 2 : 0) | (twist ? 4 : 0));
            double maxdepth = 0.0;
            int tcount = 0;
            const V3<T> hroll = hload(h, 0), htan = hload(h, 1), htw = hload(h, 2);
            const int nloop = spill ? (te - tb) : ncache;
            for (int qi = 0; qi < nloop; ++qi) {
                int tri;
                double as, dist;
                const double* W;
                if (!spill) {
                    tri = ctri[qi];
                    as = cas[qi];
                    dist = cdist[qi];
                    W = tris.world + 16 * (size_t)tri;
                } else {
                    tri = tris.ttri[tb + qi];
                    if (tris.body[tri] != b || !pt_may_touch(tris.tf, tri, pq)) continue;
                    W = tris.world + 16 * (size_t)tri;
                    as = tri_area_scale_n<T>(W, it.p, it.rad, dist);
                    if (as <= 0.0) continue;
                }
                const double depthd = it.rad - dist;
                if (dist <= 0.0 || depthd <= 0.0) continue;
                PtTri pr;
                pt_triangle_load_n<T>(m, it, bd, W, as, dist, hroll, htan, htw, pr);
                bF = bF + pr.pf;
                bT = bT + pr.ptq;
                rec[0] += pr.rf.x; rec[1] += pr.rf.y; rec[2] += pr.rf.z;
                rec[3] += pr.bt.x; rec[4] += pr.bt.y; rec[5] += pr.bt.z;
                rec[8] += pr.rf.z;
                ++tcount;
                maxdepth = fmax(maxdepth, depthd);
                if (outd) {
                    outd[0] += pr.pf.x; outd[1] += pr.pf.y; outd[2] += pr.pf.z;
                    outd[3] += pr.ptq.x; outd[4] += pr.ptq.y; outd[5] += pr.ptq.z;
                    for (int gq = 0; gq < 6; ++gq) {
                        outd[6 + 3 * gq] += pr.v[gq].x; outd[7 + 3 * gq] += pr.v[gq].y; outd[8 + 3 * gq] += pr.v[gq].z;
                    }
                    outd[24] = fmax(outd[24], depthd);
                }
            }
            rec[6] = (double)tcount;
            rec[7] = maxdepth;
            pt_microstate_n(m, it, bd, mn, mc, md, tot, cvt<double>(hload(h, 1)), cvt<double>(hload(h, 2)), rec + 10);
        }
        hb.hw[ci] = bhw;
        double* pr = ct.pt_res + 6 * (size_t)ci;
        pr[0] = bF.x; pr[1] = bF.y; pr[2] = bF.z; pr[3] = bT.x; pr[4] = bT.y; pr[5] = bT.z;
    }
    block_add(k.bover, bover);
    block_max(k.bhigh, bhigh);
}

// ------------------------------------------------------ PT, warp per item
// The lanes share the triangles of the item's cell; the per-manifold work
// (history update, microstate) is computed by every lane alike and written
// by lane 0.  Sums are taken in triangle order, each term fetched from its
// lane by shuffles, so every lane holds totals bit-identical to the serial
// loops of k_pt_thread.
//
// An FP64 warp instruction costs the same with one active lane as with 32,
// so the warp first compacts the cell's triangles that pass the FP32 test
// (in triangle order) and runs the FP64 area and law over that list, 32 at
// a time: one pass for any realistic contact instead of one per 32 cell
// triangles.  A list longer than the per-warp cache takes the uncompacted
// loops (same sums, recomputed areas).
constexpr int kPtTriCache = 128;  // per-warp candidate list: triangle, (area scale, distance)
// Two warps per block.  With few items (at most `pair_items`, the blocks that
// are resident at once) the block takes one item: warp 0 runs the law and
// hands each manifold's normal, centre, distance, area and updated history
// to warp 1 through shared memory, and warp 1 computes the microstate while
// warp 0 runs the per-triangle loads -- two FP64 chains on two of the SM's
// sub-partitions instead of one after the other.  With more items each warp
// takes items of its own and computes its microstates itself.
constexpr int kPtWarpBlock = 64;
// Blocks of k_pt_warp resident on one SM (255 registers a thread): the
// paired mode's item limit per SM.
constexpr int kPtPairBlocksPerSm = 4;

__device__ __forceinline__ V3<double> shfl3(V3<double> v, int src)
{
    return mk(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
              __shfl_sync(0xffffffffu, v.z, src));
}

// What the microstate of one manifold needs from the law (pt_microstate).
struct PtMicroIn {
    double mn[3], mc[3], th[3], twh[3], md, tot;
    int on;
};
// The block's two warps meet here once per (item, body) in paired mode
// (each warp reconverged first; named barrier 1, 64 threads).
__device__ __forceinline__ void pt_pair_barrier()
{
    __syncwarp();
    asm volatile("barrier.sync 1, 64;" ::: "memory");
}

template <typename TC, typename T>
__global__ void __launch_bounds__(kPtWarpBlock) k_pt_warp(Comps c, Owners o, Recs r, const SceneC* __restrict__ sc, Tris tris,
                                                 Bodies bodies, Hist<T> hb, Contacts<TC> ct, Counters k, double dt_eff,
                                                 int pair_items)
{
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int W = kPtWarpBlock / 32;
    __shared__ double2 s_ad[W][kPtTriCache];
    __shared__ int s_tri[W][kPtTriCache];
    __shared__ PtMicroIn s_mi[2];
    const int step = *k.step;
    const int total = *ct.pt_ctotal_ptr;
    if (total > k.pt_warp_items) return;
    const StepTape tape = tape_at(ct.tape);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    // paired: one item per block, warp 1 the observer (uniform over the grid)
    const bool paired = total <= pair_items;
    const int first = paired ? (int)blockIdx.x : (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int stride = paired ? (int)gridDim.x : (int)((gridDim.x * blockDim.x) >> 5);
    int bover = 0, bhigh = 0;
    int par = 0;  // the hand-over buffer of the next (item, body)
    for (int item = first; item < total; item += stride) {
        const int t = ct.pt_clist[item];
        const int4 meta = r.meta[t];
        const int ci = meta.x;
        const SceneC& S = sc[meta.w];
        if (paired && wib == 1) {
            // the observer: one hand-over per body, in the law warp's order
            const double rad = r.pos[t].w;
            const double mass = o.mass[meta.y];
            for (int j = 0; j < S.body_count; ++j) {
                pt_pair_barrier();
                const PtMicroIn& mi = s_mi[par];
                par ^= 1;
                if (!mi.on || lane != 0) continue;
                PtItem it;
                it.rad = rad;
                it.mass = mass;
                it.ev = mk(c.vx[ci], c.vy[ci], c.vz[ci]);
                const PtBody bd = pt_body(bodies, S.body_begin + j);
                double* rec = ct.pt_body + ((size_t)item * ct.nbs + j) * kPtRecord;
                pt_microstate(S.pt, it, bd, mk(mi.mn[0], mi.mn[1], mi.mn[2]), mk(mi.mc[0], mi.mc[1], mi.mc[2]), mi.md,
                              mi.tot, mk(mi.th[0], mi.th[1], mi.th[2]), mk(mi.twh[0], mi.twh[1], mi.twh[2]), rec + 10);
            }
            continue;
        }
        const PtItem it = pt_item(c, o, r, t, ci, meta.y, dt_eff);
        const int lin = r.cell[t].w;
        const int tb = tris.tcell_start[lin];
        const int te = min(tris.tcell_start[lin + 1], tris.capacity);
        V3<double> bF = mk(0.0, 0.0, 0.0), bT = mk(0.0, 0.0, 0.0);
        int bhw = hb.hw[ci];
        const PtProbe pq = pt_probe(it.p, it.rad);
        for (int j = 0; j < S.body_count; ++j) {
            const int b = S.body_begin + j;
            double* rec = ct.pt_body + ((size_t)item * ct.nbs + j) * kPtRecord;
            for (int f = lane; f < kPtRecord; f += 32) rec[f] = 0.0;
            double* outd = ct.pt_out ? ct.pt_out + ((size_t)item * ct.nbs + j) * 25 : nullptr;
            if (outd) for (int f = lane; f < 25; f += 32) outd[f] = 0.0;
            // candidates of body b: the cell's triangles that pass the FP32
            // test, in triangle order
            int ncand = 0;
            for (int e0 = tb; e0 < te; e0 += 32) {
                const int e = e0 + lane;
                int tri = 0;
                bool cand = false;
                if (e < te) {
                    tri = tris.ttri[e];
                    cand = tris.body[tri] == b && pt_may_touch(tris.tf, tri, pq);
                }
                const unsigned m = __ballot_sync(FULL, cand);
                const int at = ncand + __popc(m & ((1u << lane) - 1u));
                if (cand && at < kPtTriCache) s_tri[wib][at] = tri;
                ncand += __popc(m);
            }
            __syncwarp();
            const bool listed = ncand <= kPtTriCache;
            // the lane's triangle of the chunk starting at k0: from the list,
            // or (unlisted) the cell entry filtered again
            auto lane_tri = [&](int k0, int& tri) -> bool {
                if (listed) {
                    if (k0 + lane >= ncand) return false;
                    tri = s_tri[wib][k0 + lane];
                    return true;
                }
                const int e = tb + k0 + lane;
                if (e >= te) return false;
                tri = tris.ttri[e];
                return tris.body[tri] == b && pt_may_touch(tris.tf, tri, pq);
            };
            const int span = listed ? ncand : te - tb;
            // pass 1: manifold sums (:1154-1183); the triangles with a share
            // are kept in order for the adjoint tape
            double tot = 0.0, wd = 0.0;
            V3<double> wn = mk(0.0, 0.0, 0.0), wc = mk(0.0, 0.0, 0.0);
            int ttri[kPbTris];
            int tn = 0;
            for (int k0 = 0; k0 < span; k0 += 32) {
                double as = 0.0, dist = 0.0;
                int tri = 0;
                if (lane_tri(k0, tri)) {
                    as = tri_area_scale<T>(tris.world + 16 * (size_t)tri, it.p, it.rad, dist);
                    if (listed) s_ad[wib][k0 + lane] = make_double2(as, dist);
                }
                unsigned msk = __ballot_sync(FULL, as > 0.0);
                while (msk) {
                    const int src = __ffs(msk) - 1;
                    msk &= msk - 1;
                    const double a_ = __shfl_sync(FULL, as, src), d_ = __shfl_sync(FULL, dist, src);
                    const int t_ = __shfl_sync(FULL, tri, src);
                    if (tape.pb) {
                        if (tn < kPbTris) ttri[tn] = t_;
                        ++tn;
                    }
                    const double* Wt = tris.world + 16 * (size_t)t_;
                    const V3<double> out = mk(Wt[12], Wt[13], Wt[14]);
                    const V3<double> ce = it.p - out * d_;
                    tot += a_;
                    wn = wn + out * (-a_);
                    wc = wc + ce * a_;
                    wd += d_ * a_;
                }
            }
            // in paired mode every (item, body) hands a record to the observer
            // warp, an empty one where there is no manifold
            auto hand_over = [&](bool on, V3<double> mn, V3<double> mc, double md, const T* h) {
                if (!paired) return;
                if (lane == 0) {
                    PtMicroIn& mi = s_mi[par];
                    mi.on = on ? 1 : 0;
                    if (on) {
                        const V3<double> th = cvt<double>(hload(h, 1)), twh = cvt<double>(hload(h, 2));
                        mi.mn[0] = mn.x; mi.mn[1] = mn.y; mi.mn[2] = mn.z;
                        mi.mc[0] = mc.x; mi.mc[1] = mc.y; mi.mc[2] = mc.z;
                        mi.th[0] = th.x; mi.th[1] = th.y; mi.th[2] = th.z;
                        mi.twh[0] = twh.x; mi.twh[1] = twh.y; mi.twh[2] = twh.z;
                        mi.md = md;
                        mi.tot = tot;
                    }
                }
                pt_pair_barrier();
                par ^= 1;
            };
            if (tot <= 0.0) {
                hand_over(false, wn, wc, wd, nullptr);
                continue;
            }
            const V3<double> mn = normalized(wn);
            const V3<double> mc = wc * (1.0 / tot);
            const double md = wd / tot;
            int slot = 0;
            bool fresh = false;
            if (lane == 0) slot = acquire(hb, kBSlots, ci, (uint64_t)(j + 1), step, bhw, bhigh, &fresh);
            slot = __shfl_sync(FULL, slot, 0);
            bhw = __shfl_sync(FULL, bhw, 0);
            if (slot < 0) {
                if (lane == 0) ++bover;
                hand_over(false, mn, mc, md, nullptr);
                continue;
            }
            T* hv = hb.val + ((size_t)ci * kBSlots + slot) * kHV;
            T h[9];
            hv_load(hv, h);
            if (tape.pb && lane == 0) tape_pb(tape, ci, b, slot, fresh, h, ttri, tn, false);
            const PtBody bd = pt_body(bodies, b);
            const MatC& m = S.pt;
            bool slide = false, twist = false;
            pt_manifold_history<T>(m, it, bd, mn, mc, md, dt_eff, h, slide, twist);
            if (lane == 0) hv_store(hv, h);
            hand_over(true, mn, mc, md, h);
            // pass 2: per-triangle loads, the terms summed in triangle order
            double maxdepth = 0.0;
            int tcount = 0;
            V3<double> rF = mk(0.0, 0.0, 0.0), rT = mk(0.0, 0.0, 0.0);
            double rFz = 0.0;
            const LawC<T> lc = law_constants<T>(m, T(it.mass), T(it.rad));
            const V3<T> hroll = hload(h, 0), htan = hload(h, 1), htw = hload(h, 2);
            for (int k0 = 0; k0 < span; k0 += 32) {
                double as = 0.0, dist = 0.0;
                int tri = 0;
                if (listed) {
                    if (k0 + lane < ncand) {
                        tri = s_tri[wib][k0 + lane];
                        const double2 ad = s_ad[wib][k0 + lane];
                        as = ad.x;
                        dist = ad.y;
                    }
                } else if (lane_tri(k0, tri)) {
                    as = tri_area_scale<T>(tris.world + 16 * (size_t)tri, it.p, it.rad, dist);
                }
                const double depthd = it.rad - dist;
                const bool on = as > 0.0 && dist > 0.0 && depthd > 0.0;
                PtTri pr;
                if (on) pt_triangle_load<T>(m, lc, it, bd, tris.world + 16 * (size_t)tri, as, dist, hroll, htan, htw, pr);
                unsigned msk = __ballot_sync(FULL, on);
                while (msk) {
                    const int src = __ffs(msk) - 1;
                    msk &= msk - 1;
                    const V3<double> pf_ = shfl3(pr.pf, src), ptq_ = shfl3(pr.ptq, src);
                    const V3<double> rf_ = shfl3(pr.rf, src), bt_ = shfl3(pr.bt, src);
                    const double dd_ = __shfl_sync(FULL, depthd, src);
                    bF = bF + pf_;
                    bT = bT + ptq_;
                    rF = rF + rf_;
                    rT = rT + bt_;
                    rFz += rf_.z;
                    ++tcount;
                    maxdepth = fmax(maxdepth, dd_);
                    if (outd) {
                        // optional per-particle detail, accumulated by lane 0
                        V3<double> v_[6];
#pragma unroll
                        for (int gq = 0; gq < 6; ++gq) v_[gq] = shfl3(pr.v[gq], src);
                        if (lane == 0) {
                            outd[0] += pf_.x; outd[1] += pf_.y; outd[2] += pf_.z;
                            outd[3] += ptq_.x; outd[4] += ptq_.y; outd[5] += ptq_.z;
#pragma unroll
                            for (int gq = 0; gq < 6; ++gq) {
                                outd[6 + 3 * gq] += v_[gq].x; outd[7 + 3 * gq] += v_[gq].y; outd[8 + 3 * gq] += v_[gq].z;
                            }
                            outd[24] = fmax(outd[24], dd_);
                        }
                    }
                }
            }
            if (lane == 0) {
                rec[0] = rF.x; rec[1] = rF.y; rec[2] = rF.z;
                rec[3] = rT.x; rec[4] = rT.y; rec[5] = rT.z;
                rec[6] = (double)tcount;
                rec[7] = maxdepth;
                rec[8] = rFz;
                rec[9] = (double)(1 | (slide ? 2 : 0) | (twist ? 4 : 0));
                if (!paired)
                    pt_microstate(m, it, bd, mn, mc, md, tot, cvt<double>(hload(h, 1)), cvt<double>(hload(h, 2)),
                                  rec + 10);
            }
            __syncwarp();
        }
        if (lane == 0) {
            hb.hw[ci] = bhw;
            double* pr = ct.pt_res + 6 * (size_t)ci;
            pr[0] = bF.x; pr[1] = bF.y; pr[2] = bF.z; pr[3] = bT.x; pr[4] = bT.y; pr[5] = bT.z;
        }
    }
    block_add(k.bover, bover);
    block_max(k.bhigh, bhigh);
}

// --------------------------------------------------------------- owner sum
// Per owner: the reference's accumulators (:1082-1094, 1211-1220) and the
// acceleration / Euler equations (src/cuda/cuda_particle_backend.cu:71-101).
// Euler's equations of an owner (src/cuda/cuda_particle_backend.cu:71-101):
// the world-frame torque TT rotated into the body frame, the angular
// acceleration in the body frame.  The gyroscopic terms vanish for isotropic
// inertia (the flag is precomputed); the general case is kept out of line so
// its FP64 work is not issued for spheres.
__device__ __noinline__ void euler_aniso_f64(Owners o, int i, double tx, double ty, double tz)
{
    const double Ix = o.ix[i], Iy = o.iy[i], Iz = o.iz[i];
    const double wx = o.wx[i], wy = o.wy[i], wz = o.wz[i];
    o.awx[i] = (tx - (Iz - Iy) * wz * wy) * o.inv_ix[i];
    o.awy[i] = (ty - (Ix - Iz) * wx * wz) * o.inv_iy[i];
    o.awz[i] = (tz - (Iy - Ix) * wy * wx) * o.inv_iz[i];
}
__device__ __forceinline__ void euler_f64(Owners o, int i, V3<double> TT)
{
    const double qw = o.qw[i], qx = o.qx[i], qy = o.qy[i], qz = o.qz[i];
    const double tx = (1.0 - 2.0 * (qy * qy + qz * qz)) * TT.x + 2.0 * (qx * qy + qw * qz) * TT.y + 2.0 * (qx * qz - qw * qy) * TT.z;
    const double ty = 2.0 * (qx * qy - qw * qz) * TT.x + (1.0 - 2.0 * (qx * qx + qz * qz)) * TT.y + 2.0 * (qy * qz + qw * qx) * TT.z;
    const double tz = 2.0 * (qx * qz + qw * qy) * TT.x + 2.0 * (qy * qz - qw * qx) * TT.y + (1.0 - 2.0 * (qx * qx + qy * qy)) * TT.z;
    if (o.iso[i]) {
        o.awx[i] = tx * o.inv_ix[i];
        o.awy[i] = ty * o.inv_iy[i];
        o.awz[i] = tz * o.inv_iz[i];
        return;
    }
    euler_aniso_f64(o, i, tx, ty, tz);
}
// Mixed form: the rotation and Euler's equations in FP32, like the
// per-contact arithmetic they follow; the result is stored in FP64.
__device__ __noinline__ void euler_aniso_f32(Owners o, int i, float tx, float ty, float tz)
{
    const float ix = f32_rn(o.inv_ix[i]), iy = f32_rn(o.inv_iy[i]), iz = f32_rn(o.inv_iz[i]);
    const float wx = f32_rn(o.wx[i]), wy = f32_rn(o.wy[i]), wz = f32_rn(o.wz[i]);
    const float fx = f32_rn(o.ix[i]), fy = f32_rn(o.iy[i]), fz = f32_rn(o.iz[i]);
    o.awx[i] = f64_of((tx - (fz - fy) * wz * wy) * ix);
    o.awy[i] = f64_of((ty - (fx - fz) * wx * wz) * iy);
    o.awz[i] = f64_of((tz - (fy - fx) * wy * wx) * iz);
}
__device__ __forceinline__ void euler_f32(Owners o, int i, V3<float> Tq)
{
    const float qw = f32_rn(o.qw[i]), qx = f32_rn(o.qx[i]), qy = f32_rn(o.qy[i]), qz = f32_rn(o.qz[i]);
    const float tx = (1.f - 2.f * (qy * qy + qz * qz)) * Tq.x + 2.f * (qx * qy + qw * qz) * Tq.y +
                     2.f * (qx * qz - qw * qy) * Tq.z;
    const float ty = 2.f * (qx * qy - qw * qz) * Tq.x + (1.f - 2.f * (qx * qx + qz * qz)) * Tq.y +
                     2.f * (qy * qz + qw * qx) * Tq.z;
    const float tz = 2.f * (qx * qz + qw * qy) * Tq.x + 2.f * (qy * qz - qw * qx) * Tq.y +
                     (1.f - 2.f * (qx * qx + qy * qy)) * Tq.z;
    if (o.iso[i]) {
        const float ii = o.inv_i_f[i];
        o.awx[i] = f64_of(tx * ii); o.awy[i] = f64_of(ty * ii); o.awz[i] = f64_of(tz * ii);
        return;
    }
    euler_aniso_f32(o, i, tx, ty, tz);
}

// Mixed form, one sphere per owner, no force outputs: the particle rows are
// summed in FP32 (as in the general path), the translational total in FP64;
// a torque with only particle terms goes to the FP32 Euler step without a
// round trip through FP64.  The wall and body terms, when present, are added
// in FP64 in the general path's order.
template <typename T>
__device__ __forceinline__ void owner_sum_sphere_f32(Owners o, Contacts<T> ct, int i)
{
    const int cnt = ct.cnt[i];
    V3<float> sf = mk(0.f, 0.f, 0.f), st = mk(0.f, 0.f, 0.f);
    for (int q = 0; q < cnt; ++q) {
        const float* rr = reinterpret_cast<const float*>(ct.res) + 6 * ((size_t)q * o.n + i);
        sf = sf + mk(rr[0], rr[1], rr[2]);
        st = st + mk(rr[3], rr[4], rr[5]);
    }
    const V3<double> fF = mk(o.mg[3 * (size_t)i], o.mg[3 * (size_t)i + 1], o.mg[3 * (size_t)i + 2]);
    V3<double> cF = cvt<double>(sf);
    V3<double> TF = cF + (o.ugx ? fF + mk(o.ugx[i], o.ugy[i], o.ugz[i]) : fF);
    const bool wall = ct.wflag[i] != 0;
    const int pk = ct.pt_index[i];
    V3<float> Tq = st;
    if (wall || pk >= 0) {
        V3<double> wF = mk(0.0, 0.0, 0.0), wT = wF, bF = wF, bT = wF;
        if (wall) {
            const double* wr = ct.wres + 6 * (size_t)i;
            wF = mk(wr[0], wr[1], wr[2]);
            wT = mk(wr[3], wr[4], wr[5]);
        }
        if (pk >= 0) {
            const double* pr = ct.pt_res + 6 * (size_t)i;
            bF = mk(pr[0], pr[1], pr[2]);
            bT = mk(pr[3], pr[4], pr[5]);
        }
        const V3<double> cT = cvt<double>(st);
        TF = TF + (wall ? (pk >= 0 ? wF + bF : wF) : bF);
        Tq = cvt<float>(wall ? (pk >= 0 ? cT + (wT + bT) : cT + wT) : cT + bT);
    }
    const double im = o.inv_mass[i];
    o.ax[i] = TF.x * im; o.ay[i] = TF.y * im; o.az[i] = TF.z * im;
    euler_f32(o, i, Tq);
}

template <typename T>
__global__ void __launch_bounds__(256, kOwnerSumMinBlocks<T>) k_owner_sum(Comps c, Owners o, const SceneC* __restrict__ sc, Contacts<T> ct, int outputs, double* fc,
                            double* ff, double* fw, double* ft)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= o.n) return;
    if constexpr (sizeof(T) == sizeof(float)) {
        if (c.sphere && !outputs) {
            owner_sum_sphere_f32(o, ct, i);
            return;
        }
    }
    // field force m*g (precomputed per owner, the same products as
    // :1090-1094) plus universal gravitation when enabled
    V3<double> fF = mk(o.mg[3 * (size_t)i], o.mg[3 * (size_t)i + 1], o.mg[3 * (size_t)i + 2]);
    if (o.ugx) fF = fF + mk(o.ugx[i], o.ugy[i], o.ugz[i]);
    V3<double> cF = mk(0.0, 0.0, 0.0), cT = cF, wF = cF, wT = cF, bF = cF, bT = cF;
    bool any_wall = false, any_body = false;
    const int c0 = c.sphere ? i : c.ostart[i], c1 = c.sphere ? i + 1 : c.ostart[i + 1];
    for (int ci = c0; ci < c1; ++ci) {
        const int cnt = ct.cnt[ci];
        if constexpr (sizeof(T) == sizeof(double)) {
            for (int q = 0; q < cnt; ++q) {
                const T* rr = ct.res + 6 * ((size_t)q * c.n + ci);
                cF = cF + mk((double)rr[0], (double)rr[1], (double)rr[2]);
                cT = cT + mk((double)rr[3], (double)rr[4], (double)rr[5]);
            }
        } else {
            // mixed form: the per-contact rows are FP32; their sum stays FP32
            // and enters the FP64 totals once per component.
            V3<float> sf = mk(0.f, 0.f, 0.f), st = mk(0.f, 0.f, 0.f);
            for (int q = 0; q < cnt; ++q) {
                const float* rr = reinterpret_cast<const float*>(ct.res) + 6 * ((size_t)q * c.n + ci);
                sf = sf + mk(rr[0], rr[1], rr[2]);
                st = st + mk(rr[3], rr[4], rr[5]);
            }
            if (cnt) {
                cF = cF + cvt<double>(sf);
                cT = cT + cvt<double>(st);
            }
        }
        if (ct.wflag[ci]) {
            const double* wr = ct.wres + 6 * (size_t)ci;
            wF = wF + mk(wr[0], wr[1], wr[2]);
            wT = wT + mk(wr[3], wr[4], wr[5]);
            any_wall = true;
        }
        const int pk = ct.pt_index[ci];
        if (pk >= 0) {
            const double* pr = ct.pt_res + 6 * (size_t)ci;
            bF = bF + mk(pr[0], pr[1], pr[2]);
            bT = bT + mk(pr[3], pr[4], pr[5]);
            any_body = true;
        }
    }
    // total = (contact + field) + (wall + body) (:1215-1217); zero terms are
    // skipped, which leaves every sum unchanged
    const V3<double> wb = any_wall ? (any_body ? wF + bF : wF) : bF;
    const V3<double> TF = (any_wall || any_body) ? (cF + fF) + wb : cF + fF;
    const V3<double> TT = any_wall ? (any_body ? cT + (wT + bT) : cT + wT) : (any_body ? cT + bT : cT);
    if (outputs) {
        double* a = fc + 6 * (size_t)i; a[0] = cF.x; a[1] = cF.y; a[2] = cF.z; a[3] = cT.x; a[4] = cT.y; a[5] = cT.z;
        a = ff + 6 * (size_t)i; a[0] = fF.x; a[1] = fF.y; a[2] = fF.z; a[3] = 0.0; a[4] = 0.0; a[5] = 0.0;
        a = fw + 6 * (size_t)i; a[0] = wF.x; a[1] = wF.y; a[2] = wF.z; a[3] = wT.x; a[4] = wT.y; a[5] = wT.z;
        a = ft + 6 * (size_t)i; a[0] = TF.x; a[1] = TF.y; a[2] = TF.z; a[3] = TT.x; a[4] = TT.y; a[5] = TT.z;
        return;
    }
    const double im = o.inv_mass[i];
    o.ax[i] = TF.x * im; o.ay[i] = TF.y * im; o.az[i] = TF.z * im;
    if constexpr (sizeof(T) == sizeof(float)) euler_f32(o, i, cvt<float>(TT));
    else euler_f64(o, i, TT);
}
// ------------------------------------------------------------ body reduce
// Level 1: warps (group g, body b) reduce a contiguous range of contact
// items in order; level 2 reduces the groups in order.  Fields: [0..5] load,
// [6] triangle contacts, [7] max depth, [8] Fz, [9..15] regime counters,
// [16..37] microstate -> stored as kPtRecord + 6 doubles.
constexpr int kBodyFields = kBodyFieldCount;

// Regime counter f (9..15) of one record from its flags rec[9]
// (accumulateBodyRegimeKernel, :530-567): active, slide/twist class, slide,
// twist, both.
__device__ __forceinline__ double regime_field(int f, int st)
{
    if (!(st & 1)) return 0.0;
    const bool sl = (st & 2) != 0, tw = (st & 4) != 0;
    if (f == 9) return 1.0;
    if (f < 13) return (9 + (tw ? 3 : (sl ? 2 : 1))) == f ? 1.0 : 0.0;
    if (f == 13) return sl ? 1.0 : 0.0;
    if (f == 14) return tw ? 1.0 : 0.0;
    return (sl && tw) ? 1.0 : 0.0;
}
__device__ __forceinline__ double fold(double acc, double v, int f) { return f == 7 ? fmax(acc, v) : acc + v; }

// Level 1: one warp per (group, body); the group's contact items are taken
// in order, each lane folding one or two of the 38 body fields: loads, count,
// max depth and Fz straight from rec[0..8], the regime counters from the
// flags rec[9], the microstate from rec[10..31] of active manifolds.  A
// record is read coalesced across the lanes, four items in flight at a time.
template <typename T>
__global__ void k_body_partial(Recs r, const SceneC* __restrict__ sc, Bodies bodies, Contacts<T> ct, BodyOut bo)
{
    const int lane = threadIdx.x & 31;
    const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int b = blockIdx.y;
    if (g >= bo.groups) return;
    const int total = *ct.pt_ctotal_ptr;
    const int chunk = (total + bo.groups - 1) / bo.groups;
    const int beg = g * chunk, end = min(total, beg + chunk);
    const int bs = bodies.scene[b];
    const int j = b - sc[bs].body_begin;
    const int f1 = lane, f2 = lane + 32;
    const bool two = f2 < kBodyFields;
    // record index of each field (-1: derived from the flags)
    const int i1 = f1 < 9 ? f1 : (f1 >= 16 ? f1 - 6 : -1);
    const int i2 = two ? f2 - 6 : -1;
    double a1 = 0.0, a2 = 0.0;
    for (int i0 = beg; i0 < end; i0 += 4) {
        double v1[4], v2[4], st[4];
        bool use[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int item = i0 + q;
            use[q] = item < end && r.meta[ct.pt_clist[item]].w == bs;
            v1[q] = v2[q] = st[q] = 0.0;
            if (use[q]) {
                const double* rec = ct.pt_body + ((size_t)item * ct.nbs + j) * kPtRecord;
                st[q] = rec[9];
                if (i1 >= 0) v1[q] = rec[i1];
                if (i2 >= 0) v2[q] = rec[i2];
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (!use[q]) continue;
            const int sq = (int)st[q];
            const double c1 = f1 < 9 ? v1[q] : (f1 < 16 ? regime_field(f1, sq) : ((sq & 1) ? v1[q] : 0.0));
            a1 = fold(a1, c1, f1);
            if (two && (sq & 1)) a2 += v2[q];
        }
    }
    double* out = bo.partial + ((size_t)b * bo.groups + g) * kBodyFields;
    out[f1] = a1;
    if (two) out[f2] = a2;
}

// Level 2: one block per (field, body); thread k folds the groups k, k +
// 256, ... in order, then a fixed-shape tree over the threads.
__global__ void k_body_final(BodyOut bo, int interval)
{
    const int f = blockIdx.x, b = blockIdx.y;
    __shared__ double sh[256];
    double acc = 0.0;
    const double* p = bo.partial + (size_t)b * bo.groups * kBodyFields + f;
    for (int g = threadIdx.x; g < bo.groups; g += blockDim.x) acc = fold(acc, p[(size_t)g * kBodyFields], f);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = fold(sh[threadIdx.x], sh[threadIdx.x + w], f);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    acc = sh[0];
    bo.result[(size_t)b * kBodyFields + f] = acc;
    if (interval) {
        if (f >= 9 && f < 9 + kRegime) bo.reg_int[b * kRegime + (f - 9)] += (unsigned long long)acc;
        if (f >= 16) bo.micro_int[b * kMicro + (f - 16)] += acc;
        if (b == 0 && f == 0) *bo.native_steps += 1ull;
    }
}

// ------------------------------------------------ body output assembly
template <typename T>
__global__ void k_body_outputs(Comps c, Owners o, Bodies bodies, const SceneC* __restrict__ sc, Contacts<T> ct,
                               double* bp, double* bd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (i >= o.n) return;
    double acc[25];
    for (int f = 0; f < 25; ++f) acc[f] = 0.0;
    const int s = o.scene[i];
    if (bodies.scene[b] == s && ct.pt_out) {
        const int j = b - sc[s].body_begin;
        const int c0 = c.sphere ? i : c.ostart[i], c1 = c.sphere ? i + 1 : c.ostart[i + 1];
        for (int ci = c0; ci < c1; ++ci) {
            const int pk = ct.pt_index[ci];
            if (pk < 0) continue;
            const double* src = ct.pt_out + ((size_t)pk * ct.nbs + j) * 25;
            for (int f = 0; f < 24; ++f) acc[f] += src[f];
            acc[24] = fmax(acc[24], src[24]);
        }
    }
    if (bp) for (int f = 0; f < 6; ++f) bp[((size_t)b * o.n + i) * 6 + f] = acc[f];
    if (bd) for (int f = 0; f < 19; ++f) bd[((size_t)b * o.n + i) * 19 + f] = acc[6 + f];
}

inline int blocks(int n, int b) { return (n + b - 1) / b; }

}  // namespace

template <typename T>
void launch_gather_vel(const Comps& c, const Owners& o, const Grid& g, const Recs& r, double dt_eff, int sm_count,
                       int bps, cudaStream_t s)
{
    k_gather_vel<T><<<sm_count * bps, 256, 0, s>>>(c, o, g, r, dt_eff);
}

void launch_gather_geom(const Comps& c, const Owners& o, const Grid& g, const Recs& r, int sm_count, int bps,
                        const Counters& k, cudaStream_t s)
{
    k_gather_geom<<<sm_count * bps, 256, 0, s>>>(c, o, g, r, k);
}

template <typename T, typename TB>
void launch_contacts(const Comps& c, const Owners& o, const Grid& g, const Recs& r, const SceneC* sc, const Walls& w,
                     const Tris& t, const Bodies& b, Hist<T> hp, Hist<T> hw, Hist<TB> hb, Contacts<T> ct,
                     const Counters& k, double dt_eff, int block, int sm_count, cudaStream_t s, int stage)
{
    (void)block;
    if (stage & 2) {
        const int nb = blocks(c.n, 128);
        k_sweep<T><<<k.sweep_bps > 0 ? std::min(nb, sm_count * k.sweep_bps) : nb, 128, 0, s>>>(g, r, sc, hp, ct, k, c.n);
        if (ct.tape.pp) k_tape_pp<T><<<sm_count * 8, 256, 0, s>>>(r, hp, ct, k);
    }
    if ((stage & 1) && w.count > 0) {
        k_walls_probe<T><<<blocks(c.n, 256), 256, 0, s>>>(c, o, sc, w, hw, k, ct.wflag, ct.wlist);
        k_walls_law<T><<<sm_count * 4, 128, 0, s>>>(c, o, sc, w, hw, ct, k, dt_eff);
    }
    if (stage & 4) k_pp_law<T><<<sm_count * (k.pp_bps > 0 ? k.pp_bps : 16), 256, 0, s>>>(r, sc, hp, ct, k, dt_eff, g.nscenes);
    if ((stage & 8) && t.nt > 0 && b.nb > 0) {
        if (c.n <= kPtWideTileComps)
            k_pt_items<TB, kPtItemTileWide><<<std::max(1, std::min(ct.pt_scan.max_tiles, sm_count * 2)),
                                              kPtItemTileWide, 0, s>>>(g, r, t, hb, k, ct.pt_clist, ct.pt_index,
                                                                       ct.pt_ctotal_ptr, ct.pt_scan, g.err);
        else
            k_pt_items<TB, kPtItemTile><<<std::max(1, std::min(ct.pt_scan.max_tiles, sm_count * 8)), kPtItemTile, 0,
                                          s>>>(g, r, t, hb, k, ct.pt_clist, ct.pt_index, ct.pt_ctotal_ptr,
                                               ct.pt_scan, g.err);
    }
    if ((stage & 16) && t.nt > 0 && b.nb > 0) {
        k_pt_warp<T, TB><<<sm_count * 32, kPtWarpBlock, 0, s>>>(c, o, r, sc, t, b, hb, ct, k, dt_eff,
                                                             sm_count * kPtPairBlocksPerSm);
        k_pt_thread<T, TB><<<sm_count * 4, 128, 0, s>>>(c, o, r, sc, t, b, hb, ct, k, dt_eff);
    }
}

template <typename T>
void launch_owner_sum(const Comps& c, const Owners& o, const SceneC* sc, Contacts<T> ct, bool outputs, double* fc,
                      double* ff, double* fw, double* ft, cudaStream_t s)
{
    k_owner_sum<T><<<blocks(o.n, 256), 256, 0, s>>>(c, o, sc, ct, outputs ? 1 : 0, fc, ff, fw, ft);
}

template <typename T>
void launch_body_reduce(const Recs& r, const SceneC* sc, const Bodies& b, Contacts<T> ct, BodyOut bo, bool interval,
                        cudaStream_t s)
{
    if (b.nb <= 0) return;
    k_body_partial<T><<<dim3((bo.groups + 3) / 4, b.nb), 128, 0, s>>>(r, sc, b, ct, bo);
    k_body_final<<<dim3(kBodyFields, b.nb), 256, 0, s>>>(bo, interval ? 1 : 0);
}

template <typename T>
void launch_body_outputs(const Comps& c, const Owners& o, const Bodies& b, const SceneC* sc, Contacts<T> ct,
                         double* bp, double* bd, cudaStream_t s)
{
    if (b.nb <= 0) return;
    k_body_outputs<T><<<dim3(blocks(o.n, 128), b.nb), 128, 0, s>>>(c, o, b, sc, ct, bp, bd);
}

#define DEM_INSTANTIATE(T)                                                                                            \
    template void launch_gather_vel<T>(const Comps&, const Owners&, const Grid&, const Recs&, double, int, int,       \
                                       cudaStream_t);                                                                 \
    template void launch_contacts<T, double>(const Comps&, const Owners&, const Grid&, const Recs&, const SceneC*,   \
                                             const Walls&, const Tris&, const Bodies&, Hist<T>, Hist<T>,             \
                                             Hist<double>, Contacts<T>, const Counters&, double, int, int,            \
                                             cudaStream_t, int);                                                     \
    template void launch_owner_sum<T>(const Comps&, const Owners&, const SceneC*, Contacts<T>, bool, double*,       \
                                      double*, double*, double*, cudaStream_t);                                       \
    template void launch_body_reduce<T>(const Recs&, const SceneC*, const Bodies&, Contacts<T>, BodyOut, bool,       \
                                        cudaStream_t);                                                                \
    template void launch_body_outputs<T>(const Comps&, const Owners&, const Bodies&, const SceneC*, Contacts<T>,     \
                                         double*, double*, cudaStream_t);

DEM_INSTANTIATE(double)
DEM_INSTANTIATE(float)
template void launch_contacts<float, float>(const Comps&, const Owners&, const Grid&, const Recs&, const SceneC*,
                                            const Walls&, const Tris&, const Bodies&, Hist<float>, Hist<float>,
                                            Hist<float>, Contacts<float>, const Counters&, double, int, int,
                                            cudaStream_t, int);

}  // namespace demgb
