// dem_device.cuh -- device math and contact laws of the GB300 DEM engine.
//
// The laws restate the reference's constitutive model
// (src/cuda/cuda_contact_backend.cu:245-311 history response, :319-407 disk /
// triangle overlap area, :579-706 particle-particle, :708-949 particle-triangle
// manifold, :951-1063 particle-wall).  They are templated on the arithmetic
// type T: T = double is the reference's all-FP64 method, T = float is the
// mixed-precision form in which positions, overlaps and reductions stay FP64
// and the per-contact force arithmetic and the history run in FP32.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

// Law helpers compile for the host too, so their adjoints can be checked
// against finite differences on the CPU; only the overlap predicate, which
// pins a device contraction, is device-only.
#define DEM_DEV __host__ __device__ __forceinline__

namespace demgb {

constexpr double kPi = 3.1415926535897932384626433832795;
constexpr double kGravityConstant = 6.67430e-11;
constexpr int kPSlots = 64;   // particle history slots per component
constexpr int kWSlots = 16;   // wall history slots per component
constexpr int kBSlots = 64;   // body history slots per component
constexpr int kPbTris = 12;   // triangles of one particle-body manifold the reverse mode keeps
constexpr int kRegime = 7;
constexpr int kMicro = 22;
constexpr int kPtRecord = 32;  // doubles per (PT component, body) record

template <typename T> struct V3 { T x, y, z; };

// Double to float, rounded to nearest even, on the integer pipes.  On this
// GPU every FP64 conversion issues on the FP64 unit (about two lanes per
// clock per SM, the DFMA rate), so kernels that convert many state values
// to FP32 rows were bound by it.  From the IEEE-754 formats: rebias the
// exponent in the high word (1023 - 127 = 896, i.e. 896 << 20), shift the
// high word left by 3 and bring in the top 3 bits of the low word to get
// the float's exponent and 23-bit fraction, then round on the 29 dropped
// bits (ties to even); a carry out of the fraction moves into the exponent
// as it should, up to infinity.  Results equal the hardware conversion for
// |x| >= 2^-126; smaller magnitudes (float subnormals) flush to signed zero.
// Infinities stay infinite, NaNs stay NaN.
DEM_DEV float f32_rn(double x)
{
#ifdef __CUDA_ARCH__
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
#endif
    const unsigned ahi = hi & 0x7fffffffu;
    unsigned r = ((ahi - 0x38000000u) << 3) | (lo >> 29);
    r += ((lo & 0x1fffffffu) + (r & 1u)) > 0x10000000u ? 1u : 0u;
    if (ahi < 0x38100000u) r = 0u;
    if (ahi >= 0x47f00000u) r = (ahi > 0x7ff00000u || (ahi == 0x7ff00000u && lo != 0u)) ? 0x7fc00000u : 0x7f800000u;
    r |= hi & 0x80000000u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(r);
#else
    float f;
    std::memcpy(&f, &r, sizeof f);
    return f;
#endif
}

// Float to double (exact) on the integer pipes: the exponent rebiased by 896
// and the fraction shifted into place.  Float subnormals become signed zero;
// infinities and NaNs are kept.
DEM_DEV double f64_of(float f)
{
#ifdef __CUDA_ARCH__
    const unsigned u = __float_as_uint(f);
#else
    unsigned u;
    std::memcpy(&u, &f, sizeof u);
#endif
    const unsigned sign = u & 0x80000000u, a = u & 0x7fffffffu;
    unsigned hi = sign | ((a >> 3) + 0x38000000u), lo = a << 29;
    if (a < 0x00800000u) { hi = sign; lo = 0u; }
    if (a >= 0x7f800000u) { hi = sign | 0x7ff00000u | (a > 0x7f800000u ? 0x00080000u : 0u); lo = 0u; }
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
#endif
}

template <typename T> DEM_DEV V3<T> mk(T x, T y, T z) { return {x, y, z}; }
template <typename T> DEM_DEV V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> DEM_DEV V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> DEM_DEV V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename T> DEM_DEV T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> DEM_DEV V3<T> cross(V3<T> a, V3<T> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T> DEM_DEV T norm(V3<T> a) { return sqrt(dot(a, a)); }
template <typename T> DEM_DEV V3<T> normalized(V3<T> a)
{
    const T l = norm(a);
    return l > T(1.0e-14) ? a * (T(1) / l) : mk<T>(0, 0, 0);
}
// Precision conversions, between FP64 and FP32 on the integer pipes
// (f32_rn, f64_of): on GB300 the hardware conversions issue on the FP64
// unit at the DFMA rate.
template <typename T> DEM_DEV T cv(double x) { return static_cast<T>(x); }
template <typename T> DEM_DEV T cv(float x) { return static_cast<T>(x); }
template <> DEM_DEV float cv<float>(double x) { return f32_rn(x); }
template <> DEM_DEV double cv<double>(float x) { return f64_of(x); }
template <typename T, typename S> DEM_DEV V3<T> cvt(V3<S> a) { return {cv<T>(a.x), cv<T>(a.y), cv<T>(a.z)}; }

// Overlap predicate operand with a fixed contraction pattern so the contact
// set is decided by the same bits as the oracle and the reference build:
// fma(dz, dz, fma(dy, dy, dx * dx)).
__device__ __forceinline__ double distance_squared(V3<double> d)
{
    return __fma_rn(d.z, d.z, __fma_rn(d.y, d.y, __dmul_rn(d.x, d.x)));
}

// Quat2IvDCM rotation (src/cuda/cuda_contact_backend.cu:109-116).
DEM_DEV V3<double> rot_iv(double qw, double qx, double qy, double qz, V3<double> v)
{
    return {(1.0 - 2.0 * (qy * qy + qz * qz)) * v.x + 2.0 * (qx * qy - qw * qz) * v.y + 2.0 * (qx * qz + qw * qy) * v.z,
            2.0 * (qx * qy + qw * qz) * v.x + (1.0 - 2.0 * (qx * qx + qz * qz)) * v.y + 2.0 * (qy * qz - qw * qx) * v.z,
            2.0 * (qx * qz - qw * qy) * v.x + 2.0 * (qy * qz + qw * qx) * v.y + (1.0 - 2.0 * (qx * qx + qy * qy)) * v.z};
}

// packCell (src/cuda/cuda_grid_backend.cu:19-26).
__host__ __device__ inline uint64_t pack_cell(int x, int y, int z)
{
    constexpr int bias = 1 << 20;
    constexpr uint64_t mask = (1ull << 21) - 1ull;
    return ((static_cast<uint64_t>(x + bias) & mask) << 42) | ((static_cast<uint64_t>(y + bias) & mask) << 21) |
           (static_cast<uint64_t>(z + bias) & mask);
}
__host__ __device__ inline void unpack_cell(uint64_t k, int& x, int& y, int& z)
{
    constexpr int bias = 1 << 20;
    constexpr uint64_t mask = (1ull << 21) - 1ull;
    x = static_cast<int>((k >> 42) & mask) - bias;
    y = static_cast<int>((k >> 21) & mask) - bias;
    z = static_cast<int>(k & mask) - bias;
}

// Material constants of one contact class, hoisted once per scene.  The
// logarithms and the denominators pi^2 + log^2 are the exact values the
// reference recomputes per contact (:619-626).
struct MatC {
    double kN, kS, logN, logS, denN, denS, mu, muT, muR, beta, coh, dt;
};
// The same constants rounded once to FP32 (the values the FP32 laws would
// otherwise convert per contact).
struct MatF {
    float kN, kS, logN, logS, denN, denS, mu, muT, muR, beta, coh, dt;
};

// ---------------------------------------------------------------- history
// transportTangentHistory (:245-256)
template <typename T> DEM_DEV V3<T> transport_tangent(V3<T> prev, V3<T> n)
{
    const T pn = norm(prev);
    const V3<T> proj = prev - n * dot(prev, n);
    const T qn = norm(proj);
    if (pn <= T(1.0e-30) || qn <= T(1.0e-30)) return mk<T>(0, 0, 0);
    return proj * (pn / qn);
}
// transportAxialHistory (:258-265)
template <typename T> DEM_DEV V3<T> transport_axial(V3<T> prev, V3<T> n)
{
    const T pn = norm(prev);
    if (pn <= T(1.0e-30)) return mk<T>(0, 0, 0);
    const T al = dot(prev, n);
    if (fabs(al) <= T(1.0e-30)) return mk<T>(0, 0, 0);
    return n * (al < T(0) ? -pn : pn);
}
// limitedHistoryResponseRates (:267-299).  `stored` receives the new history
// value (only meaningful when the caller stores it).
template <typename T>
DEM_DEV V3<T> limited_rates(V3<T> hrate, V3<T> rrate, T k, T c, T dt, V3<T> prev, T limit, V3<T>& stored, bool& yielded)
{
    const V3<T> delta = hrate * dt;
    const V3<T> inc = delta * k;
    const V3<T> et = inc + prev;
    const V3<T> trial = rrate * c + et;
    const T tn = norm(et);
    yielded = tn > limit;
    if (yielded) {
        V3<T> resp;
        const T dn = norm(delta);
        if (dn > T(1.0e-14)) {
            resp = et * (limit / tn);
        } else {
            const T pn = norm(prev);
            resp = pn > T(1.0e-14) ? prev * (limit / pn) : mk<T>(0, 0, 0);
        }
        stored = resp;
        return resp;
    }
    stored = prev + inc;
    return trial;
}
// wallHistoryResponse (:951-973)
template <typename T>
DEM_DEV V3<T> wall_response(V3<T> rate, T k, T c, T dt, V3<T> prev, T limit, bool check_damped, bool zero_at_zero,
                            V3<T>& stored)
{
    const V3<T> delta = rate * dt;
    const V3<T> et = prev + delta * k;
    const V3<T> st = et + rate * c;
    const T tn = norm(check_damped ? st : et);
    if (tn > limit) {
        const T dn = norm(delta);
        const V3<T> lt = check_damped ? st : et;
        const V3<T> resp = (dn > T(1.0e-14) && tn > T(1.0e-14)) ? lt * (limit / tn)
                                                                  : (zero_at_zero ? mk<T>(0, 0, 0) : prev);
        stored = resp;
        return resp;
    }
    stored = et;
    return st;
}

template <typename T> DEM_DEV V3<T> hload(const T* v, int cat) { return {v[3 * cat], v[3 * cat + 1], v[3 * cat + 2]}; }
template <typename T> DEM_DEV void hstore(T* v, int cat, V3<T> x)
{
    v[3 * cat] = x.x; v[3 * cat + 1] = x.y; v[3 * cat + 2] = x.z;
}

// Damping coefficients of the reference's restitution model (:619-632).
template <typename T> struct LawC { T kN, kS, cN, cS, kT, cT, kR, cR, brs; };
template <typename T, typename M> DEM_DEV LawC<T> law_constants(const M& m, T mred, T radius_term)
{
    LawC<T> c;
    c.kN = T(m.kN);
    c.kS = T(m.kS);
    c.cN = T(-2.0) * T(m.logN) * sqrt(c.kN * mred / T(m.denN));
    c.cS = T(-2.0) * T(m.logS) * sqrt(c.kS * mred / T(m.denS));
    c.brs = T(m.beta) * radius_term * T(m.beta) * radius_term;
    c.kT = T(2.0) * c.kS * c.brs;
    c.cT = T(2.0) * c.cS * c.brs;
    c.kR = c.kN * c.brs;
    c.cR = c.cN * c.brs;
    return c;
}

// ------------------------------------------------------------ PP contact
// particleContact (:579-706) after the overlap test and slot acquisition.
// n: unit direction i->j; erv/mrv: endpoint/midpoint velocity of j minus i;
// h: history slot values [roll, tangent, twist] updated in place.
template <typename T, typename M>
DEM_DEV void pp_law(const M& m, T dt, V3<T> n, T d, T depth, T d2, T ri, T rj, T mi, T mj, V3<T> erv, V3<T> mrv,
                    V3<T> ewi, V3<T> ewj, V3<T> mwi, V3<T> mwj, T* h, V3<T>& force, V3<T>& couple)
{
    const T mred = mi * mj / (mi + mj);
    const T rs = ri + rj;
    const T reff = ri * rj / rs;
    const LawC<T> c = law_constants<T, M>(m, mred, reff);
    V3<T> fn = n * (-c.kN * depth) + n * (c.cN * dot(erv, n));
    fn = fn + n * (T(m.coh) * T(4.0) * c.brs);
    const T li = (ri * ri - rj * rj + d2) / (T(2.0) * d);
    const T lj = d - li;
    V3<T> etv = erv - n * dot(erv, n);
    etv = etv + cross(n, ewi) * li;
    etv = etv + cross(n, ewj) * lj;
    V3<T> mtv = mrv - n * dot(mrv, n);
    mtv = mtv + cross(n, mwi) * li;
    mtv = mtv + cross(n, mwj) * lj;
    bool y;
    V3<T> st;
    const V3<T> fr = limited_rates<T>(mtv, etv, c.kS, c.cS, dt, transport_tangent(hload(h, 1), n), T(m.mu) * norm(fn),
                                      st, y);
    hstore(h, 1, st);
    const V3<T> erw = ewj - ewi, mrw = mwj - mwi;
    const V3<T> etw = n * dot(erw, n), mtw = n * dot(mrw, n);
    const V3<T> erl = erw - etw, mrl = mrw - mtw;
    const T ms = T(m.beta) * reff * norm(fn);
    const V3<T> tw = limited_rates<T>(mtw, etw, c.kT, c.cT, dt, transport_axial(hload(h, 2), n),
                                      T(m.mu) * T(m.muT) * ms, st, y);
    hstore(h, 2, st);
    const V3<T> rl = limited_rates<T>(mrl, erl, c.kR, c.cR, dt, transport_tangent(hload(h, 0), n), T(m.muR) * ms, st, y);
    hstore(h, 0, st);
    force = fn + fr;
    couple = (tw + rl) + cross(n, fr) * li;
}

// ---------------------------------------------------------- wall contact
// wallContact (:975-1063) after the slot acquisition; out = outward normal.
template <typename T, typename M>
DEM_DEV void wall_law(const M& m, T dt, V3<T> out, T depth, T r, T mass, V3<T> vel, V3<T> om, T* h, V3<T>& force,
                      V3<T>& couple)
{
    const V3<T> n = out * T(-1.0);
    const T lever = r - depth;
    const V3<T> rv = vel * T(-1.0);
    V3<T> tv = rv - n * dot(rv, n);
    tv = tv + cross(n, om) * lever;
    const V3<T> rw = om * T(-1.0);
    const V3<T> twr = n * dot(rw, n);
    V3<T> rlr = rw - twr;
    if (fabs(lever) > T(1.0e-30)) rlr = rlr + cross(n, tv) * (T(0.5) / lever);
    const LawC<T> c = law_constants<T, M>(m, mass, r);
    const V3<T> en = n * (-c.kN * depth);
    const V3<T> dn = n * (c.cN * dot(rv, n));
    const V3<T> fn = en + dn;
    const T flim = T(m.mu) * norm(fn);
    const T ms = T(m.beta) * r * norm(fn);
    V3<T> st;
    const V3<T> fr = wall_response<T>(tv, c.kS, c.cS, dt, transport_tangent(hload(h, 1), n), flim, false, false, st);
    hstore(h, 1, st);
    const V3<T> tw = wall_response<T>(twr, c.kT, c.cT, dt, transport_axial(hload(h, 2), n), T(m.mu) * T(m.muT) * ms,
                                      false, true, st);
    hstore(h, 2, st);
    const V3<T> rl = wall_response<T>(rlr, c.kR, c.cR, dt, transport_tangent(hload(h, 0), n), T(m.muR) * ms, true, true,
                                      st);
    hstore(h, 0, st);
    force = fn + fr;
    couple = (tw + rl) + cross(n, fr) * lever;
}

// ----------------------------------------------------------- disk area
// circleEdgeArea (:319-358), 2-D coordinates relative to the disk centre.
template <typename T> DEM_DEV T circle_edge_area(T ax, T ay, T bx, T by, T r)
{
    const T dx = bx - ax, dy = by - ay;
    const T aa = dx * dx + dy * dy;
    T cuts[4] = {T(0), T(1), T(0), T(0)};
    int n = 2;
    if (aa > T(1.0e-30)) {
        const T bb = T(2.0) * (ax * dx + ay * dy);
        const T cc = (ax * ax + ay * ay) - r * r;
        const T disc = bb * bb - T(4.0) * aa * cc;
        if (disc > T(0)) {
            const T root = sqrt(disc);
            const T t0 = (-bb - root) / (T(2.0) * aa);
            const T t1 = (-bb + root) / (T(2.0) * aa);
            if (t0 > T(0) && t0 < T(1)) cuts[n++] = t0;
            if (t1 > T(0) && t1 < T(1)) cuts[n++] = t1;
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            if (cuts[j] < cuts[i]) { const T tmp = cuts[i]; cuts[i] = cuts[j]; cuts[j] = tmp; }
    T area = T(0);
    for (int i = 0; i + 1 < n; ++i) {
        const T ta = cuts[i], tb = cuts[i + 1];
        const T ux = ax + dx * ta, uy = ay + dy * ta;
        const T vx = ax + dx * tb, vy = ay + dy * tb;
        const T tm = T(0.5) * (ta + tb);
        const T mx = ax + dx * tm, my = ay + dy * tm;
        const T cr = ux * vy - uy * vx;
        if (mx * mx + my * my <= r * r) area += T(0.5) * cr;
        else area += T(0.5) * r * r * atan2(cr, ux * vx + uy * vy);
    }
    return area;
}

// circleTriangleArea (:360-378).  ra, rb, rc: triangle vertices minus the
// disk centre.
template <typename T> DEM_DEV T circle_triangle_area(V3<T> normal, V3<T> ra, V3<T> rb, V3<T> rc, T r)
{
    const V3<T> axis = fabs(normal.x) < T(0.8) ? mk<T>(1, 0, 0) : mk<T>(0, 1, 0);
    const V3<T> u = normalized(cross(normal, axis));
    const V3<T> v = cross(normal, u);
    const T ax = dot(ra, u), ay = dot(ra, v), bx = dot(rb, u), by = dot(rb, v), cx = dot(rc, u), cy = dot(rc, v);
    T area = circle_edge_area<T>(ax, ay, bx, by, r) + circle_edge_area<T>(bx, by, cx, cy, r) +
             circle_edge_area<T>(cx, cy, ax, ay, r);
    area = fabs(area);
    return fmin(area, T(kPi) * r * r);
}

// World record of one triangle (transformTrianglesKernel,
// src/cuda/cuda_body_backend.cu:71-112): W[0..11] the vertices v1..v4 at
// R(q) L_k + c, W[12..14] the normal R(q) L[12..14], W[15] the circumradius of
// v2..v4 about their centroid (used only to skip disjoint pairs).  Also
// returns that centroid (g) for the FP32 prefilter copies.
DEM_DEV void tri_world(const double* L, double qw, double qx, double qy, double qz, double cx, double cy, double cz,
                       double* W, double g[3])
{
    for (int k = 0; k < 4; ++k) {
        const V3<double> p = rot_iv(qw, qx, qy, qz, mk(L[3 * k], L[3 * k + 1], L[3 * k + 2]));
        W[3 * k] = p.x + cx; W[3 * k + 1] = p.y + cy; W[3 * k + 2] = p.z + cz;
    }
    const V3<double> nn = rot_iv(qw, qx, qy, qz, mk(L[12], L[13], L[14]));
    W[12] = nn.x; W[13] = nn.y; W[14] = nn.z;
    g[0] = (W[3] + W[6] + W[9]) * (1.0 / 3.0);
    g[1] = (W[4] + W[7] + W[10]) * (1.0 / 3.0);
    g[2] = (W[5] + W[8] + W[11]) * (1.0 / 3.0);
    double r2 = 0.0;
    for (int k = 1; k < 4; ++k) {
        const double dx = W[3 * k] - g[0], dy = W[3 * k + 1] - g[1], dz = W[3 * k + 2] - g[2];
        r2 = fmax(r2, dx * dx + dy * dy + dz * dz);
    }
    W[15] = sqrt(r2) * (1.0 + 1e-12) + 1e-15;
}

// Whether the contact disk (centre at the common origin of the in-plane
// vertex offsets ra, rb, rc; squared radius c2) lies beyond one of the
// triangle's edge lines, on the side away from the triangle, by more than
// its radius: then disk and triangle are disjoint.  With s the signed
// doubled area of (centre, a, b) and S that of the triangle, the centre is
// beyond edge ab when s and S differ in sign, at the distance |s| / |b - a|.
// The margin, 1e-6 of the squared distances, is far above the rounding of
// these products.
DEM_DEV bool disk_beyond_an_edge(V3<double> n, V3<double> ra, V3<double> rb, V3<double> rc, double c2)
{
    const V3<double> e0 = rb - ra, e1 = rc - rb, e2 = ra - rc;
    const double S = dot(cross(e0, rc - ra), n);
    const double s0 = dot(cross(ra, rb), n), s1 = dot(cross(rb, rc), n), s2 = dot(cross(rc, ra), n);
    const double m = c2 * (1.0 + 1.0e-6);
    return (s0 * S < 0.0 && s0 * s0 > m * dot(e0, e0)) || (s1 * S < 0.0 && s1 * s1 > m * dot(e1, e1)) ||
           (s2 * S < 0.0 && s2 * s2 > m * dot(e2, e2));
}

// The contact disk of a sphere (centre p, radius r) on the plane of the
// world triangle W: the sphere's distance above the plane along the normal,
// the disk's squared radius and the vertex offsets from its centre (the
// same arithmetic as the start of tri_area_scale64 below).
struct TriDisk {
    V3<double> n, ra, rb, rc;
    double dist, c2;
};
// The tests of bodyTriangleAreaScale (:380-407) that need no edge sum: false
// when the scale is certainly 0 -- the sphere not strictly above the plane
// within its radius, or disk and triangle disjoint (disk centre farther from
// the triangle's centroid than the disk radius plus the triangle's
// circumradius about it, W[15], or beyond an edge by more than the disk
// radius).  For disjoint shapes the reference's edge sum cancels to rounding
// noise, far below its 1e-12 threshold, so the scale is 0 either way.
DEM_DEV bool tri_disk(const double* W, V3<double> p, double r, TriDisk& d)
{
    d.n = mk(W[12], W[13], W[14]);
    const V3<double> a = mk(W[3], W[4], W[5]);
    d.dist = dot(d.n, p - a);
    if (d.dist <= 0.0) return false;
    d.c2 = r * r - d.dist * d.dist;
    if (d.c2 <= 1.0e-30) return false;
    const V3<double> ce = p - d.n * d.dist;
    d.ra = a - ce;
    d.rb = mk(W[6], W[7], W[8]) - ce;
    d.rc = mk(W[9], W[10], W[11]) - ce;
    const V3<double> cen = (d.ra + d.rb + d.rc) * (1.0 / 3.0);
    const double reach = (sqrt(d.c2) + W[15]) * (1.0 + 1e-9);
    if (dot(cen, cen) > reach * reach) return false;
    return !disk_beyond_an_edge(d.n, d.ra, d.rb, d.rc, d.c2);
}

// bodyTriangleAreaScale (:380-407) in FP64: the share of the contact disk of
// a sphere (centre p, radius r) that lies on the world triangle W, and the
// sphere's distance above the triangle's plane (dist, along the normal).
DEM_DEV double tri_area_scale64(const double* W, V3<double> p, double r, double& dist)
{
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
    const double area = circle_triangle_area<double>(n, ra, rb, rc, sqrt(c2));
    if (area <= 0.0) return 0.0;
    const double sc = fmin(1.0, area / (kPi * c2));
    return sc > 1.0e-12 ? sc : 0.0;
}

}  // namespace demgb
