// Central-difference check of the step adjoints in dem_adjoint.cuh, on the
// host.  For random inputs (both capped and uncapped history branches) and
// random output adjoints lo, the VJP must match d(lo . f)/dx component by
// component.  Prints one line per check and "ALL OK" when every check
// passes.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../dem_mbd_cuda_gb300/csrc/dem_adjoint.cuh"

using namespace demgb;

static std::mt19937_64 rng(20261203);
static double U(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }
static D3 R3(double s) { return mk(U(-s, s), U(-s, s), U(-s, s)); }

struct Mat {
    double kN, mu, logN, logS, muT, muR, beta, coh;
    MatC c() const
    {
        MatC m;
        m.kN = kN; m.kS = 2.0 * kN / 7.0; m.logN = logN; m.logS = logS;
        m.denN = kPi * kPi + logN * logN; m.denS = kPi * kPi + logS * logS;
        m.mu = mu; m.muT = muT; m.muR = muR; m.beta = beta; m.coh = coh; m.dt = 0.0;
        return m;
    }
};

static int failures = 0;
static void check(const char* what, double an, double fd, double rel = 1e-5, double abs = 1e-9)
{
    const double err = fabs(an - fd), scale = fmax(fabs(an), fabs(fd));
    const bool ok = err <= rel * scale + abs;
    if (!ok) ++failures;
    if (!ok) printf("FAIL %-28s analytic % .9e  fd % .9e\n", what, an, fd);
}

// ---- particle law: all outputs as one vector
static std::vector<double> pp_fwd(const Mat& mt, double dt, const PPIn& in)
{
    const MatC m = mt.c();
    const double d2 = dot(in.delta, in.delta), d = sqrt(d2);
    const D3 n = in.delta * (1.0 / d);
    double h[9];
    memcpy(h, in.h, sizeof h);
    D3 f, cpl;
    pp_law<double, MatC>(m, dt, n, d, in.ri + in.rj - d, d2, in.ri, in.rj, in.mi, in.mj, in.erv, in.mrv, in.ewi, in.ewj,
                         in.mwi, in.mwj, h, f, cpl);
    std::vector<double> o = {f.x, f.y, f.z, cpl.x, cpl.y, cpl.z};
    for (int k = 0; k < 9; ++k) o.push_back(h[k]);
    return o;
}
static double dotv(const std::vector<double>& a, const std::vector<double>& b)
{
    double s = 0.0;
    for (size_t k = 0; k < a.size(); ++k) s += a[k] * b[k];
    return s;
}

static void pp_case(double hscale, const char* tag)
{
    Mat mt = {U(5e4, 2e5), U(0.2, 0.6), log(U(0.3, 0.8)), log(U(0.3, 0.8)), U(0.05, 0.3), U(0.02, 0.2), 0.5, U(0, 5)};
    const double dt = 1e-5;
    PPIn in;
    in.ri = U(1.8e-3, 2.2e-3); in.rj = U(1.8e-3, 2.2e-3);
    const D3 dir = normalized(R3(1.0));
    in.delta = dir * (in.ri + in.rj - U(1e-6, 2e-5));
    in.mi = 2500 * 4.18879 * in.ri * in.ri * in.ri; in.mj = 2500 * 4.18879 * in.rj * in.rj * in.rj;
    in.erv = R3(0.1); in.mrv = R3(0.1); in.ewi = R3(5); in.ewj = R3(5); in.mwi = R3(5); in.mwj = R3(5);
    for (int k = 0; k < 9; ++k) in.h[k] = U(-hscale, hscale);
    std::vector<double> lo(15);
    for (auto& x : lo) x = U(-1, 1);
    PPAdj a;
    memset(&a, 0, sizeof a);
    MatGrad g = {0, 0, 0, 0, 0, 0};
    pp_law_vjp(mt.c(), dt, in, mk(lo[0], lo[1], lo[2]), mk(lo[3], lo[4], lo[5]), lo.data() + 6, a, g);
    auto fdv = [&](auto set, double x0, double h) {
        PPIn p = in;
        set(p, x0 + h);
        const double fp = dotv(lo, pp_fwd(mt, dt, p));
        set(p, x0 - h);
        const double fm = dotv(lo, pp_fwd(mt, dt, p));
        return (fp - fm) / (2 * h);
    };
    char name[64];
    D3* vin[] = {&in.delta, &in.erv, &in.mrv, &in.ewi, &in.ewj, &in.mwi, &in.mwj};
    D3* vad[] = {&a.delta, &a.erv, &a.mrv, &a.ewi, &a.ewj, &a.mwi, &a.mwj};
    const char* vn[] = {"delta", "erv", "mrv", "ewi", "ewj", "mwi", "mwj"};
    for (int v = 0; v < 7; ++v)
        for (int c = 0; c < 3; ++c) {
            const size_t off = (char*)vin[v] - (char*)&in + c * sizeof(double);
            const double x0 = *(double*)((char*)&in + off);
            const double h = 1e-4 * fmax(fabs(x0), v == 0 ? 1e-3 : 1e-2);
            const double fd = fdv([off](PPIn& p, double x) { *(double*)((char*)&p + off) = x; }, x0, h);
            const double an = c == 0 ? vad[v]->x : (c == 1 ? vad[v]->y : vad[v]->z);
            snprintf(name, sizeof name, "pp %s %s[%d]", tag, vn[v], c);
            check(name, an, fd);
        }
    for (int k = 0; k < 9; ++k) {
        const double x0 = in.h[k], h = 1e-4 * fmax(fabs(x0), 1e-4);
        const double fd = fdv([k](PPIn& p, double x) { p.h[k] = x; }, x0, h);
        snprintf(name, sizeof name, "pp %s h[%d]", tag, k);
        check(name, a.h[k], fd);
    }
    // material parameters
    auto fdm = [&](double Mat::*f, double h) {
        Mat p = mt;
        p.*f = mt.*f + h;
        const double fp = dotv(lo, pp_fwd(p, dt, in));
        p.*f = mt.*f - h;
        const double fm = dotv(lo, pp_fwd(p, dt, in));
        return (fp - fm) / (2 * h);
    };
    snprintf(name, sizeof name, "pp %s kN", tag); check(name, g.kN, fdm(&Mat::kN, 1e-6 * mt.kN));
    snprintf(name, sizeof name, "pp %s mu", tag); check(name, g.mu, fdm(&Mat::mu, 1e-6));
    snprintf(name, sizeof name, "pp %s logN", tag); check(name, g.logN, fdm(&Mat::logN, 1e-6));
    snprintf(name, sizeof name, "pp %s logS", tag); check(name, g.logS, fdm(&Mat::logS, 1e-6));
    snprintf(name, sizeof name, "pp %s muT", tag); check(name, g.muT, fdm(&Mat::muT, 1e-6));
    snprintf(name, sizeof name, "pp %s muR", tag); check(name, g.muR, fdm(&Mat::muR, 1e-6));
}

// ---- wall law
struct PWIn {
    D3 out, p, o, vel, om;
    double r, mass, h[9];
};
static std::vector<double> pw_fwd(const Mat& mt, double dt, const PWIn& in)
{
    const MatC m = mt.c();
    const double depth = in.r - dot(in.p - in.o, in.out);
    double h[9];
    memcpy(h, in.h, sizeof h);
    D3 f, cpl;
    wall_law<double, MatC>(m, dt, in.out, depth, in.r, in.mass, in.vel, in.om, h, f, cpl);
    std::vector<double> o = {f.x, f.y, f.z, cpl.x, cpl.y, cpl.z};
    for (int k = 0; k < 9; ++k) o.push_back(h[k]);
    return o;
}
static void pw_case(double hscale, const char* tag)
{
    Mat mt = {U(5e4, 2e5), U(0.2, 0.6), log(U(0.3, 0.8)), log(U(0.3, 0.8)), U(0.05, 0.3), U(0.02, 0.2), 0.5, 0.0};
    const double dt = 1e-5;
    PWIn in;
    in.out = normalized(R3(1.0));
    in.o = R3(0.1);
    in.r = U(1.8e-3, 2.2e-3);
    in.p = in.o + in.out * (in.r - U(1e-6, 2e-5)) + cross(in.out, R3(0.01));
    in.mass = 2500 * 4.18879 * in.r * in.r * in.r;
    in.vel = R3(0.1); in.om = R3(5);
    for (int k = 0; k < 9; ++k) in.h[k] = U(-hscale, hscale);
    std::vector<double> lo(15);
    for (auto& x : lo) x = U(-1, 1);
    PWAdj a;
    memset(&a, 0, sizeof a);
    MatGrad g = {0, 0, 0, 0, 0, 0};
    const double depth = in.r - dot(in.p - in.o, in.out);
    pw_law_vjp(mt.c(), dt, in.out, depth, in.r, in.mass, in.vel, in.om, in.h, mk(lo[0], lo[1], lo[2]),
               mk(lo[3], lo[4], lo[5]), lo.data() + 6, a, g);
    char name[64];
    D3* vin[] = {&in.p, &in.vel, &in.om};
    D3* vad[] = {&a.p, &a.vel, &a.om};
    const char* vn[] = {"p", "vel", "om"};
    for (int v = 0; v < 3; ++v)
        for (int c = 0; c < 3; ++c) {
            double* x = (c == 0 ? &vin[v]->x : (c == 1 ? &vin[v]->y : &vin[v]->z));
            const double x0 = *x, h = v == 0 ? 1e-8 : 1e-4 * fmax(fabs(x0), 1e-2);
            *x = x0 + h; const double fp = dotv(lo, pw_fwd(mt, dt, in));
            *x = x0 - h; const double fm = dotv(lo, pw_fwd(mt, dt, in));
            *x = x0;
            const double an = c == 0 ? vad[v]->x : (c == 1 ? vad[v]->y : vad[v]->z);
            snprintf(name, sizeof name, "pw %s %s[%d]", tag, vn[v], c);
            check(name, an, (fp - fm) / (2 * h));
        }
    for (int k = 0; k < 9; ++k) {
        const double x0 = in.h[k], h = 1e-4 * fmax(fabs(x0), 1e-4);
        in.h[k] = x0 + h; const double fp = dotv(lo, pw_fwd(mt, dt, in));
        in.h[k] = x0 - h; const double fm = dotv(lo, pw_fwd(mt, dt, in));
        in.h[k] = x0;
        snprintf(name, sizeof name, "pw %s h[%d]", tag, k);
        check(name, a.h[k], (fp - fm) / (2 * h));
    }
    auto fdm = [&](double Mat::*f, double h) {
        Mat p = mt;
        p.*f = mt.*f + h; const double fp = dotv(lo, pw_fwd(p, dt, in));
        p.*f = mt.*f - h; const double fm = dotv(lo, pw_fwd(p, dt, in));
        return (fp - fm) / (2 * h);
    };
    snprintf(name, sizeof name, "pw %s kN", tag); check(name, g.kN, fdm(&Mat::kN, 1e-6 * mt.kN));
    snprintf(name, sizeof name, "pw %s mu", tag); check(name, g.mu, fdm(&Mat::mu, 1e-6));
    snprintf(name, sizeof name, "pw %s logN", tag); check(name, g.logN, fdm(&Mat::logN, 1e-6));
    snprintf(name, sizeof name, "pw %s logS", tag); check(name, g.logS, fdm(&Mat::logS, 1e-6));
    snprintf(name, sizeof name, "pw %s muT", tag); check(name, g.muT, fdm(&Mat::muT, 1e-6));
    snprintf(name, sizeof name, "pw %s muR", tag); check(name, g.muR, fdm(&Mat::muR, 1e-6));
}

// ---- rotations and quaternion maps
static void quat_cases()
{
    char name[64];
    for (int t = 0; t < 20; ++t) {
        double q[4] = {U(-1, 1), U(-1, 1), U(-1, 1), U(-1, 1)};
        const D3 v = R3(3), lo = R3(1);
        double lq[4] = {0, 0, 0, 0};
        D3 lv = z3();
        rotq_vjp(q, v, lo, lq, lv);
        for (int k = 0; k < 4; ++k) {
            double qp[4], qm[4];
            memcpy(qp, q, sizeof q); memcpy(qm, q, sizeof q);
            qp[k] += 1e-6; qm[k] -= 1e-6;
            const double fd = (dot(lo, rotq(qp, v)) - dot(lo, rotq(qm, v))) / 2e-6;
            snprintf(name, sizeof name, "rotq q[%d]", k); check(name, lq[k], fd);
        }
        double lq2[4] = {0, 0, 0, 0};
        D3 lt = z3();
        rotq_t_vjp(q, v, lo, lq2, lt);
        for (int k = 0; k < 4; ++k) {
            double qp[4], qm[4];
            memcpy(qp, q, sizeof q); memcpy(qm, q, sizeof q);
            qp[k] += 1e-6; qm[k] -= 1e-6;
            const double fd = (dot(lo, rotq_t(qp, v)) - dot(lo, rotq_t(qm, v))) / 2e-6;
            snprintf(name, sizeof name, "rotq_t q[%d]", k); check(name, lq2[k], fd);
        }
        {
            D3 vp = v; vp.y += 1e-6; D3 vm = v; vm.y -= 1e-6;
            check("rotq_t t[1]", lt.y, (dot(lo, rotq_t(q, vp)) - dot(lo, rotq_t(q, vm))) / 2e-6);
            check("rotq v[1]", lv.y, (dot(lo, rotq(q, vp)) - dot(lo, rotq(q, vm))) / 2e-6);
        }
        // quat derivative and normalisation
        const double l4[4] = {U(-1, 1), U(-1, 1), U(-1, 1), U(-1, 1)};
        double lqd[4] = {0, 0, 0, 0};
        D3 lw = z3();
        quatd_vjp(q, v, l4, lqd, lw);
        auto qdot = [&](const double* qq, D3 ww) {
            double o[4];
            quatd(qq, ww, o);
            return o[0] * l4[0] + o[1] * l4[1] + o[2] * l4[2] + o[3] * l4[3];
        };
        for (int k = 0; k < 4; ++k) {
            double qp[4], qm[4];
            memcpy(qp, q, sizeof q); memcpy(qm, q, sizeof q);
            qp[k] += 1e-6; qm[k] -= 1e-6;
            snprintf(name, sizeof name, "quatd q[%d]", k); check(name, lqd[k], (qdot(qp, v) - qdot(qm, v)) / 2e-6);
        }
        {
            D3 vp = v; vp.z += 1e-6; D3 vm = v; vm.z -= 1e-6;
            check("quatd w[2]", lw.z, (qdot(q, vp) - qdot(q, vm)) / 2e-6);
        }
        double ln[4] = {0, 0, 0, 0};
        normq_vjp(q, l4, ln);
        auto nq = [&](const double* qq) {
            const double n = sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
            return (qq[0] * l4[0] + qq[1] * l4[1] + qq[2] * l4[2] + qq[3] * l4[3]) / n;
        };
        for (int k = 0; k < 4; ++k) {
            double qp[4], qm[4];
            memcpy(qp, q, sizeof q); memcpy(qm, q, sizeof q);
            qp[k] += 1e-6; qm[k] -= 1e-6;
            snprintf(name, sizeof name, "normq q[%d]", k); check(name, ln[k], (nq(qp) - nq(qm)) / 2e-6);
        }
    }
}


// ---- particle-triangle manifold (area shares, manifold, history, loads)
// A hexagonal fan of six triangles in the body's z = 0 plane (normal +z),
// the sphere above it in the body frame; `off` moves the contact disk from
// the fan's centre (several triangles) toward its rim (arcs cut by the rim).
struct PTCase {
    double L[6][15];
    PTIn in;
};
static std::vector<double> pt_vec(const Mat& mt, double dt, const PTIn& in)
{
    PTOut o;
    pt_manifold_fwd(mt.c(), dt, in, o);
    std::vector<double> v = {o.pf.x, o.pf.y, o.pf.z, o.ptq.x, o.ptq.y, o.ptq.z, o.rf.x, o.rf.y, o.rf.z,
                             o.bt.x, o.bt.y, o.bt.z};
    for (int k = 0; k < 9; ++k) v.push_back(o.h[k]);
    return v;
}
static void pt_case(double hscale, double off, double apex, const char* tag)
{
    Mat mt = {U(5e4, 2e5), U(0.2, 0.6), log(U(0.3, 0.8)), log(U(0.3, 0.8)), U(0.05, 0.3), U(0.02, 0.2), 0.5, U(0, 5)};
    const double dt = 1e-5, R = 3e-3;
    PTCase pc;
    for (int k = 0; k < 6; ++k) {
        const double a0 = k * kPi / 3, a1 = (k + 1) * kPi / 3;
        // apex > 0 raises the fan's centre: a pyramid of six tilted faces
        const double v2[3] = {0, 0, apex}, v3[3] = {R * cos(a0), R * sin(a0), 0}, v4[3] = {R * cos(a1), R * sin(a1), 0};
        double* L = pc.L[k];
        for (int i = 0; i < 3; ++i) {
            L[i] = (v2[i] + v3[i] + v4[i]) / 3; L[3 + i] = v2[i]; L[6 + i] = v3[i]; L[9 + i] = v4[i];
        }
        const D3 nn = normalized(cross(mk(v3[0] - v2[0], v3[1] - v2[1], v3[2] - v2[2]),
                                       mk(v4[0] - v2[0], v4[1] - v2[1], v4[2] - v2[2])));
        L[12] = nn.x; L[13] = nn.y; L[14] = nn.z;
    }
    PTIn& in = pc.in;
    in.rad = U(1.8e-3, 2.2e-3);
    in.mass = 2500 * 4.18879 * in.rad * in.rad * in.rad;
    const double q0[4] = {U(-1, 1), U(-1, 1), U(-1, 1), U(-1, 1)};
    const double qn = sqrt(q0[0] * q0[0] + q0[1] * q0[1] + q0[2] * q0[2] + q0[3] * q0[3]);
    for (int k = 0; k < 4; ++k) in.q[k] = q0[k] / qn;
    in.c = R3(0.05);
    const double ang = U(0, 2 * kPi);
    const D3 pb = mk(off * cos(ang), off * sin(ang), apex + in.rad * U(0.6, 0.9));
    in.p = in.c + rotq(in.q, pb);
    in.ev = R3(0.05); in.mv = R3(0.05); in.ew = R3(5); in.mw = R3(5);
    in.V = R3(0.05); in.w = R3(3);
    in.ntri = 6;
    for (int k = 0; k < 6; ++k) in.L[k] = pc.L[k];
    // histories as contacts carry them: roll and tangent in the contact
    // plane, twist along the normal (away from the axial transport's sign
    // flip, a jump of the reference's map where the twist history is
    // perpendicular to the normal)
    // per channel (roll, tangent, twist) a magnitude well inside its cap
    const double hs[3] = {5e-3 * hscale, 0.5 * hscale, 5e-3 * hscale};
    {
        const D3 nb = rotq(in.q, mk(0.0, 0.0, 1.0));
        for (int ch = 0; ch < 2; ++ch) {
            D3 v = R3(1.0);
            v = normalized(v - nb * dot(v, nb)) * (hs[ch] * U(0.5, 1.0));
            in.h[3 * ch] = v.x; in.h[3 * ch + 1] = v.y; in.h[3 * ch + 2] = v.z;
        }
        const D3 tw = nb * (U(0.5, 1.0) * hs[2] * (U(0, 1) < 0.5 ? -1.0 : 1.0)) + R3(0.1 * hs[2]);
        in.h[6] = tw.x; in.h[7] = tw.y; in.h[8] = tw.z;
    }
    std::vector<double> lo(21);
    for (auto& x : lo) x = U(-1, 1);
    PTAdj a;
    memset(&a, 0, sizeof a);
    MatGrad g = {0, 0, 0, 0, 0, 0};
    pt_manifold_vjp(mt.c(), dt, in, mk(lo[0], lo[1], lo[2]), mk(lo[3], lo[4], lo[5]), mk(lo[6], lo[7], lo[8]),
                    mk(lo[9], lo[10], lo[11]), lo.data() + 12, a, g);
    // fourth-order central differences: the history transports curve on
    // the scale of the history's own (small, elastic) magnitude
    auto fdv = [&](size_t off_b, double x0, double h) {
        PTIn p = in;
        auto at = [&](double x) {
            *(double*)((char*)&p + off_b) = x;
            return dotv(lo, pt_vec(mt, dt, p));
        };
        return (at(x0 - 2 * h) - 8 * at(x0 - h) + 8 * at(x0 + h) - at(x0 + 2 * h)) / (12 * h);
    };
    char name[64];
    D3* vin[] = {&in.p, &in.ev, &in.mv, &in.ew, &in.mw, &in.c, &in.V, &in.w};
    D3* vad[] = {&a.p, &a.ev, &a.mv, &a.ew, &a.mw, &a.c, &a.V, &a.w};
    const char* vn[] = {"p", "ev", "mv", "ew", "mw", "c", "V", "w"};
    // steps where central differences settle: positions (m), velocities (m/s), spins (rad/s)
    const double step[] = {1e-9, 1e-6, 1e-6, 1e-4, 1e-4, 1e-9, 1e-6, 1e-4};
    for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 3; ++c) {
            const size_t ob = (char*)vin[v] - (char*)&in + c * sizeof(double);
            const double x0 = *(double*)((char*)&in + ob);
            const double h = step[v];
            const double an = c == 0 ? vad[v]->x : (c == 1 ? vad[v]->y : vad[v]->z);
            snprintf(name, sizeof name, "pt %s %s[%d]", tag, vn[v], c);
            check(name, an, fdv(ob, x0, h), 1e-4);
        }
    for (int k = 0; k < 4; ++k) {
        const size_t ob = (char*)&in.q[k] - (char*)&in;
        snprintf(name, sizeof name, "pt %s q[%d]", tag, k);
        check(name, a.q[k], fdv(ob, in.q[k], 1e-6), 1e-4);
    }
    for (int k = 0; k < 9; ++k) {
        const size_t ob = (char*)&in.h[k] - (char*)&in;
        snprintf(name, sizeof name, "pt %s h[%d]", tag, k);
        check(name, a.h[k], fdv(ob, in.h[k], 1e-3 * hs[k / 3]), 1e-4, 1e-7);
    }
    auto fdm = [&](double Mat::*f, double h) {
        Mat p = mt;
        p.*f = mt.*f + h;
        const double fp = dotv(lo, pt_vec(p, dt, in));
        p.*f = mt.*f - h;
        const double fm = dotv(lo, pt_vec(p, dt, in));
        return (fp - fm) / (2 * h);
    };
    snprintf(name, sizeof name, "pt %s kN", tag); check(name, g.kN, fdm(&Mat::kN, 1e-6 * mt.kN), 1e-4);
    snprintf(name, sizeof name, "pt %s mu", tag); check(name, g.mu, fdm(&Mat::mu, 1e-6), 1e-4);
    snprintf(name, sizeof name, "pt %s logN", tag); check(name, g.logN, fdm(&Mat::logN, 1e-6), 1e-4);
    snprintf(name, sizeof name, "pt %s logS", tag); check(name, g.logS, fdm(&Mat::logS, 1e-6), 1e-4);
    snprintf(name, sizeof name, "pt %s muT", tag); check(name, g.muT, fdm(&Mat::muT, 1e-6), 1e-4);
    snprintf(name, sizeof name, "pt %s muR", tag); check(name, g.muR, fdm(&Mat::muR, 1e-6), 1e-4);
}

// ---- body leapfrog: the position update into a step and its half update
struct BodyState {
    double c[3], q[4], hv[3], hw[3], hdq[4], acc[3], dom[3], F[6];
};
static std::vector<double> body_vec(const BodyState& b, const double bc[4], double dt, bool first, const double* V0,
                                    const double* W0)
{
    const double half = 0.5 * dt;
    double c[3], q[4], V[3], W[3];
    if (first) {
        for (int a = 0; a < 3; ++a) { c[a] = b.c[a]; V[a] = V0[a]; W[a] = W0[a]; }
        for (int k = 0; k < 4; ++k) q[k] = b.q[k];
    } else {
        for (int a = 0; a < 3; ++a) {
            c[a] = b.c[a] + b.hv[a] * dt; V[a] = b.hv[a] + b.acc[a] * half; W[a] = b.hw[a] + b.dom[a] * half;
        }
        double r[4];
        for (int k = 0; k < 4; ++k) r[k] = b.q[k] + b.hdq[k] * dt;
        const double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
        for (int k = 0; k < 4; ++k) q[k] = r[k] / len;
    }
    D3 acc, dom;
    body_dyn(b.F, q, mk(W[0], W[1], W[2]), bc, acc, dom);
    const double f = first ? half : dt;
    const double hv[3] = {(first ? V[0] : b.hv[0]) + acc.x * f, (first ? V[1] : b.hv[1]) + acc.y * f,
                          (first ? V[2] : b.hv[2]) + acc.z * f};
    const double hw[3] = {(first ? W[0] : b.hw[0]) + dom.x * f, (first ? W[1] : b.hw[1]) + dom.y * f,
                          (first ? W[2] : b.hw[2]) + dom.z * f};
    double g[4], r[4], hq[4], hdq[4];
    quatd(q, mk(W[0], W[1], W[2]), g);
    for (int k = 0; k < 4; ++k) r[k] = q[k] + g[k] * half;
    const double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
    for (int k = 0; k < 4; ++k) hq[k] = r[k] / len;
    quatd(hq, mk(hw[0], hw[1], hw[2]), hdq);
    std::vector<double> v;
    for (double x : c) v.push_back(x);
    for (double x : q) v.push_back(x);
    for (double x : V) v.push_back(x);
    for (double x : W) v.push_back(x);
    for (double x : hv) v.push_back(x);
    for (double x : hw) v.push_back(x);
    for (double x : hdq) v.push_back(x);
    v.push_back(acc.x); v.push_back(acc.y); v.push_back(acc.z);
    v.push_back(dom.x); v.push_back(dom.y); v.push_back(dom.z);
    return v;
}
static void body_case(bool first)
{
    const double dt = 1e-4, bc[4] = {U(0.5, 2), U(1e-3, 3e-3), U(1e-3, 3e-3), U(1e-3, 3e-3)};
    BodyState b;
    double V0[3], W0[3];
    for (int a = 0; a < 3; ++a) {
        b.c[a] = U(-0.1, 0.1); b.hv[a] = U(-0.5, 0.5); b.hw[a] = U(-3, 3); b.acc[a] = U(-5, 5); b.dom[a] = U(-20, 20);
        V0[a] = U(-0.5, 0.5); W0[a] = U(-3, 3);
    }
    double qn = 0;
    for (int k = 0; k < 4; ++k) { b.q[k] = U(-1, 1); qn += b.q[k] * b.q[k]; }
    for (int k = 0; k < 4; ++k) { b.q[k] /= sqrt(qn); b.hdq[k] = U(-2, 2); }
    for (int k = 0; k < 6; ++k) b.F[k] = U(-10, 10);
    const std::vector<double> y = body_vec(b, bc, dt, first, V0, W0);
    std::vector<double> lo(y.size());
    for (auto& x : lo) x = U(-1, 1);
    // the record of the step, and the adjoint of the state after it
    double rec[kBR], prev[kBR];
    for (int k = 0; k < 3; ++k) {
        rec[kBrC + k] = y[k]; rec[kBrV + k] = y[7 + k]; rec[kBrW + k] = y[10 + k];
        rec[kBrHV + k] = y[13 + k]; rec[kBrHW + k] = y[16 + k]; rec[kBrAcc + k] = y[23 + k]; rec[kBrDom + k] = y[26 + k];
    }
    for (int k = 0; k < 4; ++k) { rec[kBrQ + k] = y[3 + k]; rec[kBrHDQ + k] = y[19 + k]; }
    for (int k = 0; k < 6; ++k) rec[kBrF + k] = b.F[k];
    {
        // hq of the step, as the half update makes it
        double g[4], r[4];
        quatd(rec + kBrQ, ldv3(rec, kBrW), g);
        for (int k = 0; k < 4; ++k) r[k] = rec[kBrQ + k] + g[k] * 0.5 * dt;
        const double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
        for (int k = 0; k < 4; ++k) rec[kBrHQ + k] = r[k] / len;
    }
    for (int k = 0; k < 4; ++k) { prev[kBrQ + k] = b.q[k]; prev[kBrHDQ + k] = b.hdq[k]; }
    double Lb[kBL] = {};
    const int map[25] = {kBlC, kBlC + 1, kBlC + 2, kBlQ, kBlQ + 1, kBlQ + 2, kBlQ + 3, kBlV, kBlV + 1, kBlV + 2,
                         kBlW, kBlW + 1, kBlW + 2, kBlHV, kBlHV + 1, kBlHV + 2, kBlHW, kBlHW + 1, kBlHW + 2,
                         kBlHDQ, kBlHDQ + 1, kBlHDQ + 2, kBlHDQ + 3, kBlAcc, kBlAcc + 1};
    for (int k = 0; k < 25; ++k) Lb[map[k]] = lo[k];
    Lb[kBlAcc + 2] = lo[25];
    for (int k = 0; k < 3; ++k) Lb[kBlDom + k] = lo[26 + k];
    body_half_vjp(rec, bc, dt, first, Lb);
    if (!first) body_pos_vjp(prev, dt, Lb);
    auto fd = [&](double* x, double h, bool pose_v) {
        BodyState p = b;
        double V0p[3], W0p[3];
        memcpy(V0p, V0, sizeof V0p); memcpy(W0p, W0, sizeof W0p);
        double* px = pose_v ? x : (double*)((char*)&p + ((char*)x - (char*)&b));
        if (pose_v) px = x == V0 ? V0p : W0p;
        const double x0 = *px;
        (void)x0;
        auto run = [&](double d) {
            double save = *px;
            *px = save + d;
            const double f = dotv(lo, body_vec(p, bc, dt, first, V0p, W0p));
            *px = save;
            return f;
        };
        return (run(h) - run(-h)) / (2 * h);
    };
    char name[64];
    for (int k = 0; k < 6; ++k) {
        snprintf(name, sizeof name, "body%s F[%d]", first ? "0" : "", k);
        check(name, Lb[kBlF + k], fd(&b.F[k], 1e-4, false));
    }
    if (first) {
        for (int k = 0; k < 3; ++k) {
            snprintf(name, sizeof name, "body0 c[%d]", k); check(name, Lb[kBlC + k], fd(&b.c[k], 1e-3, false));
        }
        for (int k = 0; k < 4; ++k) {
            snprintf(name, sizeof name, "body0 q[%d]", k); check(name, Lb[kBlQ + k], fd(&b.q[k], 1e-6, false));
        }
        for (int k = 0; k < 3; ++k) {
            // V0 and W0 through the pose slots
            BodyState p = b;
            double Vp[3], Vm[3], Wp[3], Wm[3];
            memcpy(Vp, V0, sizeof Vp); memcpy(Vm, V0, sizeof Vm); memcpy(Wp, W0, sizeof Wp); memcpy(Wm, W0, sizeof Wm);
            Vp[k] += 1e-5; Vm[k] -= 1e-5;
            snprintf(name, sizeof name, "body0 V[%d]", k);
            check(name, Lb[kBlV + k], (dotv(lo, body_vec(p, bc, dt, true, Vp, W0)) - dotv(lo, body_vec(p, bc, dt, true, Vm, W0))) / 2e-5);
            Wp[k] += 1e-5; Wm[k] -= 1e-5;
            snprintf(name, sizeof name, "body0 W[%d]", k);
            check(name, Lb[kBlW + k], (dotv(lo, body_vec(p, bc, dt, true, V0, Wp)) - dotv(lo, body_vec(p, bc, dt, true, V0, Wm))) / 2e-5);
        }
        return;
    }
    for (int k = 0; k < 3; ++k) {
        snprintf(name, sizeof name, "body c[%d]", k); check(name, Lb[kBlC + k], fd(&b.c[k], 1e-3, false));
        snprintf(name, sizeof name, "body hv[%d]", k); check(name, Lb[kBlHV + k], fd(&b.hv[k], 1e-5, false));
        snprintf(name, sizeof name, "body hw[%d]", k); check(name, Lb[kBlHW + k], fd(&b.hw[k], 1e-5, false));
        snprintf(name, sizeof name, "body acc[%d]", k); check(name, Lb[kBlAcc + k], fd(&b.acc[k], 1e-2, false));
        snprintf(name, sizeof name, "body dom[%d]", k); check(name, Lb[kBlDom + k], fd(&b.dom[k], 1e-2, false));
    }
    for (int k = 0; k < 4; ++k) {
        snprintf(name, sizeof name, "body q[%d]", k); check(name, Lb[kBlQ + k], fd(&b.q[k], 1e-6, false));
        snprintf(name, sizeof name, "body hdq[%d]", k); check(name, Lb[kBlHDQ + k], fd(&b.hdq[k], 1e-4, false));
    }
}

int main()
{
    quat_cases();
    for (int t = 0; t < 40; ++t) {
        // history forces below the tangential cap (twist and roll capped) and
        // above every cap
        pp_case(1e-2, "elastic-t");
        pp_case(10.0, "capped");
        pw_case(1e-2, "elastic-t");
        pw_case(10.0, "capped");
    }
    // The manifold's history update and its read-only loads: a channel that
    // caps in the update sits exactly at its cap in the loads, a tie that
    // central differences cannot straddle, so these cases keep every channel
    // elastic in the update (the capped branches are the laws' own, checked
    // above).
    for (int t = 0; t < 30; ++t) {
        pt_case(1e-2, 0.5e-3, 0.0, "centre");
        pt_case(1e-2, 2.6e-3, 0.0, "rim");
        pt_case(1e-2, 0.8e-3, 0.4e-3, "bent");
        body_case(false);
        body_case(true);
    }
    if (failures) {
        printf("%d FAILED\n", failures);
        return 1;
    }
    printf("ALL OK\n");
    return 0;
}
