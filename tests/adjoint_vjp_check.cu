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
static void check(const char* what, double an, double fd)
{
    const double err = fabs(an - fd), scale = fmax(fabs(an), fabs(fd));
    const bool ok = err <= 1e-5 * scale + 1e-9;
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
    if (failures) {
        printf("%d FAILED\n", failures);
        return 1;
    }
    printf("ALL OK\n");
    return 0;
}
