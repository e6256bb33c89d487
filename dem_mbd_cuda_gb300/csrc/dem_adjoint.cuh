// dem_adjoint.cuh -- vector-Jacobian products of one step of the FP64 form.
//
// Reverse mode of the step the engine takes (the reference's leapfrog,
// src/cuda/cuda_particle_backend.cu:149-265, and its contact laws,
// src/cuda/cuda_contact_backend.cu:245-311, :579-706, :951-1063).  Each
// function recomputes the forward quantities it needs from the same inputs
// and maps the adjoints of the outputs to the adjoints of the inputs and of
// the material parameters.  Within a step the contact set is what the
// forward step found (it is held fixed); at the Coulomb, twisting and rolling
// caps the derivative is that of the branch the forward step took (a
// subgradient at the cap itself).  The functions compile for the host as well,
// so tests check them against central differences on the CPU.
#pragma once

#include "dem_device.cuh"

namespace demgb {

using D3 = V3<double>;

// Adjoints of the material constants of one contact class: kN (kS = 2 kN / 7
// is folded in), mu, log(epsN) and log(epsS) (the denominators pi^2 + log^2
// are folded in), muT, muR.
struct MatGrad {
    double kN, mu, logN, logS, muT, muR;
};

DEM_DEV D3 z3() { return mk(0.0, 0.0, 0.0); }

// ------------------------------------------------------------- primitives
// a x b: adjoint la += b x lo, lb += lo x a
DEM_DEV void cross_vjp(D3 a, D3 b, D3 lo, D3& la, D3& lb)
{
    la = la + cross(b, lo);
    lb = lb + cross(lo, a);
}
// |a|
DEM_DEV void norm_vjp(D3 a, double lo, D3& la)
{
    const double n = norm(a);
    if (n > 0.0) la = la + a * (lo / n);
}
// q / |q| (normalize_quat; the degenerate reset to identity has no adjoint)
DEM_DEV void normq_vjp(const double q[4], const double lo[4], double lq[4])
{
    const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (n2 <= 1.0e-24) return;
    const double inv = 1.0 / sqrt(n2);
    double o[4], d = 0.0;
    for (int k = 0; k < 4; ++k) { o[k] = q[k] * inv; d += o[k] * lo[k]; }
    for (int k = 0; k < 4; ++k) lq[k] += (lo[k] - o[k] * d) * inv;
}
// quat_derivative G(q, w) = 0.5 q (x) (0, w)
DEM_DEV void quatd(const double q[4], D3 w, double o[4])
{
    o[0] = 0.5 * (-q[1] * w.x - q[2] * w.y - q[3] * w.z);
    o[1] = 0.5 * (q[0] * w.x + q[2] * w.z - q[3] * w.y);
    o[2] = 0.5 * (q[0] * w.y - q[1] * w.z + q[3] * w.x);
    o[3] = 0.5 * (q[0] * w.z + q[1] * w.y - q[2] * w.x);
}
DEM_DEV void quatd_vjp(const double q[4], D3 w, const double lo[4], double lq[4], D3& lw)
{
    lq[0] += 0.5 * (lo[1] * w.x + lo[2] * w.y + lo[3] * w.z);
    lq[1] += 0.5 * (-lo[0] * w.x - lo[2] * w.z + lo[3] * w.y);
    lq[2] += 0.5 * (-lo[0] * w.y + lo[1] * w.z - lo[3] * w.x);
    lq[3] += 0.5 * (-lo[0] * w.z - lo[1] * w.y + lo[2] * w.x);
    lw.x += 0.5 * (-lo[0] * q[1] + lo[1] * q[0] + lo[2] * q[3] - lo[3] * q[2]);
    lw.y += 0.5 * (-lo[0] * q[2] - lo[1] * q[3] + lo[2] * q[0] + lo[3] * q[1]);
    lw.z += 0.5 * (-lo[0] * q[3] + lo[1] * q[2] - lo[2] * q[1] + lo[3] * q[0]);
}
// rot_iv(q, v) = R(q) v (body -> world)
DEM_DEV D3 rotq(const double q[4], D3 v) { return rot_iv(q[0], q[1], q[2], q[3], v); }
DEM_DEV void rotq_vjp(const double q[4], D3 v, D3 lo, double lq[4], D3& lv)
{
    const double qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    // lv += R^T lo
    lv.x += (1.0 - 2.0 * (qy * qy + qz * qz)) * lo.x + 2.0 * (qx * qy + qw * qz) * lo.y + 2.0 * (qx * qz - qw * qy) * lo.z;
    lv.y += 2.0 * (qx * qy - qw * qz) * lo.x + (1.0 - 2.0 * (qx * qx + qz * qz)) * lo.y + 2.0 * (qy * qz + qw * qx) * lo.z;
    lv.z += 2.0 * (qx * qz + qw * qy) * lo.x + 2.0 * (qy * qz - qw * qx) * lo.y + (1.0 - 2.0 * (qx * qx + qy * qy)) * lo.z;
    // lq += (d(R v)/dq)^T lo
    const double vx = v.x, vy = v.y, vz = v.z;
    lq[0] += lo.x * (-2.0 * qz * vy + 2.0 * qy * vz) + lo.y * (2.0 * qz * vx - 2.0 * qx * vz) +
             lo.z * (-2.0 * qy * vx + 2.0 * qx * vy);
    lq[1] += lo.x * (2.0 * qy * vy + 2.0 * qz * vz) + lo.y * (2.0 * qy * vx - 4.0 * qx * vy - 2.0 * qw * vz) +
             lo.z * (2.0 * qz * vx + 2.0 * qw * vy - 4.0 * qx * vz);
    lq[2] += lo.x * (-4.0 * qy * vx + 2.0 * qx * vy + 2.0 * qw * vz) + lo.y * (2.0 * qx * vx + 2.0 * qz * vz) +
             lo.z * (-2.0 * qw * vx + 2.0 * qz * vy - 4.0 * qy * vz);
    lq[3] += lo.x * (-4.0 * qz * vx - 2.0 * qw * vy + 2.0 * qx * vz) + lo.y * (2.0 * qw * vx - 4.0 * qz * vy + 2.0 * qy * vz) +
             lo.z * (2.0 * qx * vx + 2.0 * qy * vy);
}
// R(q)^T t (world -> body, the Euler-equation transform of the owner sum) is
// R(conj q) t
DEM_DEV D3 rotq_t(const double q[4], D3 t)
{
    const double c[4] = {q[0], -q[1], -q[2], -q[3]};
    return rotq(c, t);
}
DEM_DEV void rotq_t_vjp(const double q[4], D3 t, D3 lo, double lq[4], D3& lt)
{
    const double c[4] = {q[0], -q[1], -q[2], -q[3]};
    double lc[4] = {0.0, 0.0, 0.0, 0.0};
    rotq_vjp(c, t, lo, lc, lt);
    lq[0] += lc[0]; lq[1] -= lc[1]; lq[2] -= lc[2]; lq[3] -= lc[3];
}

// --------------------------------------------------------- history maps
DEM_DEV void transport_tangent_vjp(D3 h, D3 n, D3 lo, D3& lh, D3& ln)
{
    const double pn = norm(h);
    const double hn = dot(h, n);
    const D3 proj = h - n * hn;
    const double qn = norm(proj);
    if (pn <= 1.0e-30 || qn <= 1.0e-30) return;
    const double s = pn / qn;
    D3 lproj = lo * s;
    const double ls = dot(proj, lo);
    const double lpn = ls / qn, lqn = -ls * pn / (qn * qn);
    lproj = lproj + proj * (lqn / qn);
    lh = lh + h * (lpn / pn);
    const double nl = dot(n, lproj);
    lh = lh + (lproj - n * nl);
    ln = ln + lproj * (-hn) - h * nl;
}
DEM_DEV void transport_axial_vjp(D3 h, D3 n, D3 lo, D3& lh, D3& ln)
{
    const double pn = norm(h);
    if (pn <= 1.0e-30) return;
    const double al = dot(h, n);
    if (fabs(al) <= 1.0e-30) return;
    const double sg = al < 0.0 ? -1.0 : 1.0;
    ln = ln + lo * (sg * pn);
    lh = lh + h * (sg * dot(n, lo) / pn);
}

// limitedHistoryResponseRates (:267-299): (resp, stored) from (hrate,
// rrate, k, c, prev, limit); lr = adjoint of resp, ls = of stored.
DEM_DEV void limited_rates_vjp(D3 hrate, D3 rrate, double k, double c, double dt, D3 prev, double limit, D3 lr, D3 ls,
                               D3& lhrate, D3& lrrate, double& lk, double& lc, D3& lprev, double& llimit)
{
    const D3 delta = hrate * dt;
    const D3 inc = delta * k;
    const D3 et = inc + prev;
    const double tn = norm(et);
    D3 linc = z3();
    if (tn > limit) {
        const D3 lR = lr + ls;
        if (norm(delta) > 1.0e-14) {
            const double g = limit / tn;
            D3 let = lR * g;
            const double lg = dot(et, lR);
            llimit += lg / tn;
            const double ltn = -lg * limit / (tn * tn);
            let = let + et * (ltn / tn);
            linc = let;
            lprev = lprev + let;
        } else {
            const double pn = norm(prev);
            if (pn > 1.0e-14) {
                const double g = limit / pn;
                lprev = lprev + lR * g;
                const double lg = dot(prev, lR);
                llimit += lg / pn;
                const double lpn = -lg * limit / (pn * pn);
                lprev = lprev + prev * (lpn / pn);
            }
        }
    } else {
        linc = lr + ls;
        lprev = lprev + lr + ls;
        lrrate = lrrate + lr * c;
        lc += dot(rrate, lr);
    }
    lk += dot(delta, linc);
    lhrate = lhrate + linc * (k * dt);
}

// wallHistoryResponse (:951-973)
DEM_DEV void wall_response_vjp(D3 rate, double k, double c, double dt, D3 prev, double limit, bool check_damped,
                               bool zero_at_zero, D3 lr, D3 ls, D3& lrate, double& lk, double& lc, D3& lprev,
                               double& llimit)
{
    const D3 delta = rate * dt;
    const D3 et = prev + delta * k;
    const D3 st = et + rate * c;
    const double tn = norm(check_damped ? st : et);
    D3 let = z3();
    if (tn > limit) {
        const D3 lR = lr + ls;
        const double dn = norm(delta);
        if (dn > 1.0e-14 && tn > 1.0e-14) {
            const D3 lt = check_damped ? st : et;
            const double g = limit / tn;
            D3 llt = lR * g;
            const double lg = dot(lt, lR);
            llimit += lg / tn;
            const double ltn = -lg * limit / (tn * tn);
            llt = llt + lt * (ltn / tn);
            if (check_damped) {
                let = llt;
                lrate = lrate + llt * c;
                lc += dot(rate, llt);
            } else {
                let = llt;
            }
        } else if (!zero_at_zero) {
            lprev = lprev + lR;
        }
    } else {
        let = ls + lr;
        lrate = lrate + lr * c;
        lc += dot(rate, lr);
    }
    lprev = lprev + let;
    lk += dot(delta, let);
    lrate = lrate + let * (k * dt);
}

// Adjoints of the per-contact constants (law_constants) -> material
// adjoints.  mred and the radius term are fixed per pair.
struct LawL {
    double kN, kS, cN, cS, kT, cT, kR, cR;
};
DEM_DEV void law_constants_vjp(const MatC& m, double mred, double rterm, const LawL& l, MatGrad& g)
{
    const double brs = m.beta * rterm * m.beta * rterm;
    double lkS = l.kS + 2.0 * brs * l.kT;
    const double lcS = l.cS + 2.0 * brs * l.cT;
    double lkN = l.kN + brs * l.kR;
    const double lcN = l.cN + brs * l.cR;
    // cN = -2 logN sqrt(kN mred / denN), denN = pi^2 + logN^2
    {
        const double A = m.kN * mred / m.denN, sA = sqrt(A);
        const double lA = -m.logN * lcN / sA;
        g.logN += -2.0 * sA * lcN;
        lkN += lA * mred / m.denN;
        const double lden = -lA * m.kN * mred / (m.denN * m.denN);
        g.logN += 2.0 * m.logN * lden;
    }
    // cS = -2 logS sqrt(kS mred / denS)
    {
        const double A = m.kS * mred / m.denS, sA = sqrt(A);
        const double lA = -m.logS * lcS / sA;
        g.logS += -2.0 * sA * lcS;
        lkS += lA * mred / m.denS;
        const double lden = -lA * m.kS * mred / (m.denS * m.denS);
        g.logS += 2.0 * m.logS * lden;
    }
    g.kN += lkN + lkS * (2.0 / 7.0);
}

// --------------------------------------------------------- particle law
// Inputs of one contact side i (partner j): delta = p_j - p_i, radii,
// masses, endpoint and midpoint relative velocities (erv, mrv), world
// angular velocities (endpoint ew, midpoint mw), history h[9] before the
// step.  Output adjoints: force lF, couple lC (on i), stored history lh[9].
struct PPIn {
    D3 delta;
    double ri, rj, mi, mj;
    D3 erv, mrv, ewi, ewj, mwi, mwj;
    double h[9];
};
struct PPAdj {
    D3 delta, erv, mrv, ewi, ewj, mwi, mwj;
    double h[9];
};

DEM_DEV void pp_law_vjp(const MatC& m, double dt, const PPIn& in, D3 lF, D3 lC, const double lh_out[9], PPAdj& a,
                        MatGrad& g)
{
    // forward
    const double d2 = dot(in.delta, in.delta);
    const double d = sqrt(d2);
    const D3 n = in.delta * (1.0 / d);
    const double rs = in.ri + in.rj;
    const double depth = rs - d;
    const double mred = in.mi * in.mj / (in.mi + in.mj);
    const double reff = in.ri * in.rj / rs;
    const LawC<double> c = law_constants<double, MatC>(m, mred, reff);
    const double ervn = dot(in.erv, n);
    const double phi = -c.kN * depth + c.cN * ervn + m.coh * 4.0 * c.brs;
    const D3 fn = n * phi;
    const double A = in.ri * in.ri - in.rj * in.rj;
    const double li = (A + d2) / (2.0 * d);
    const double lj = d - li;
    const D3 X1 = cross(n, in.ewi), X2 = cross(n, in.ewj), Y1 = cross(n, in.mwi), Y2 = cross(n, in.mwj);
    const double mrvn = dot(in.mrv, n);
    const D3 etv = in.erv - n * ervn + X1 * li + X2 * lj;
    const D3 mtv = in.mrv - n * mrvn + Y1 * li + Y2 * lj;
    const D3 h0 = mk(in.h[0], in.h[1], in.h[2]), h1 = mk(in.h[3], in.h[4], in.h[5]), h2 = mk(in.h[6], in.h[7], in.h[8]);
    const D3 prev_t = transport_tangent(h1, n);
    const double fnn = norm(fn);
    const double Lt = m.mu * fnn;
    D3 st;
    bool y;
    const D3 fr = limited_rates<double>(mtv, etv, c.kS, c.cS, dt, prev_t, Lt, st, y);
    const D3 erw = in.ewj - in.ewi, mrw = in.mwj - in.mwi;
    const double erwn = dot(erw, n), mrwn = dot(mrw, n);
    const D3 etw = n * erwn, mtw = n * mrwn;
    const D3 erl = erw - etw, mrl = mrw - mtw;
    const double ms = m.beta * reff * fnn;
    const D3 prev_w = transport_axial(h2, n);
    const double Lw = m.mu * m.muT * ms;
    const D3 prev_r = transport_tangent(h0, n);
    const double Lr = m.muR * ms;

    // reverse
    D3 ln = z3(), lfn = lF, lfr = lF;
    double lli = 0.0, llj = 0.0, ld = 0.0, ld2 = 0.0, ldepth = 0.0;
    LawL ll = {0, 0, 0, 0, 0, 0, 0, 0};
    // couple = (tw + rl) + cross(n, fr) li
    const D3 lX = lC * li;
    lli += dot(cross(n, fr), lC);
    cross_vjp(n, fr, lX, ln, lfr);
    // roll channel
    D3 lmrl = z3(), lerl = z3(), lpr = z3();
    double lLr = 0.0;
    limited_rates_vjp(mrl, erl, c.kR, c.cR, dt, prev_r, Lr, lC, mk(lh_out[0], lh_out[1], lh_out[2]), lmrl, lerl, ll.kR,
                      ll.cR, lpr, lLr);
    // twist channel
    D3 lmtw = z3(), letw = z3(), lpw = z3();
    double lLw = 0.0;
    limited_rates_vjp(mtw, etw, c.kT, c.cT, dt, prev_w, Lw, lC, mk(lh_out[6], lh_out[7], lh_out[8]), lmtw, letw, ll.kT,
                      ll.cT, lpw, lLw);
    // tangential channel
    D3 lmtv = z3(), letv = z3(), lpt = z3();
    double lLt = 0.0;
    limited_rates_vjp(mtv, etv, c.kS, c.cS, dt, prev_t, Lt, lfr, mk(lh_out[3], lh_out[4], lh_out[5]), lmtv, letv, ll.kS,
                      ll.cS, lpt, lLt);
    // limits
    double lms = m.muR * lLr + m.mu * m.muT * lLw;
    g.muR += ms * lLr;
    g.mu += m.muT * ms * lLw + fnn * lLt;
    g.muT += m.mu * ms * lLw;
    const double lfnn = m.beta * reff * lms + m.mu * lLt;
    norm_vjp(fn, lfnn, lfn);
    // transports
    D3 lh0 = z3(), lh1 = z3(), lh2 = z3();
    transport_tangent_vjp(h0, n, lpr, lh0, ln);
    transport_axial_vjp(h2, n, lpw, lh2, ln);
    transport_tangent_vjp(h1, n, lpt, lh1, ln);
    // rolling and twisting rates: erl = erw - n (erw.n), etw = n (erw.n)
    D3 lerw = z3(), lmrw = z3();
    {
        const double nl = dot(n, lerl);
        lerw = lerw + lerl - n * nl;
        ln = ln + lerl * (-erwn) - erw * nl;
        const double nt = dot(n, letw);
        ln = ln + letw * erwn + erw * nt;
        lerw = lerw + n * nt;
    }
    {
        const double nl = dot(n, lmrl);
        lmrw = lmrw + lmrl - n * nl;
        ln = ln + lmrl * (-mrwn) - mrw * nl;
        const double nt = dot(n, lmtw);
        ln = ln + lmtw * mrwn + mrw * nt;
        lmrw = lmrw + n * nt;
    }
    a.ewj = a.ewj + lerw; a.ewi = a.ewi - lerw;
    a.mwj = a.mwj + lmrw; a.mwi = a.mwi - lmrw;
    // etv = erv - n (erv.n) + X1 li + X2 lj
    {
        const double nl = dot(n, letv);
        a.erv = a.erv + letv - n * nl;
        ln = ln + letv * (-ervn) - in.erv * nl;
        lli += dot(X1, letv);
        llj += dot(X2, letv);
        cross_vjp(n, in.ewi, letv * li, ln, a.ewi);
        cross_vjp(n, in.ewj, letv * lj, ln, a.ewj);
    }
    {
        const double nl = dot(n, lmtv);
        a.mrv = a.mrv + lmtv - n * nl;
        ln = ln + lmtv * (-mrvn) - in.mrv * nl;
        lli += dot(Y1, lmtv);
        llj += dot(Y2, lmtv);
        cross_vjp(n, in.mwi, lmtv * li, ln, a.mwi);
        cross_vjp(n, in.mwj, lmtv * lj, ln, a.mwj);
    }
    // lj = d - li, li = (A + d2) / (2 d)
    ld += llj;
    lli -= llj;
    ld2 += lli / (2.0 * d);
    ld -= lli * (A + d2) / (2.0 * d * d);
    // fn = n phi
    ln = ln + lfn * phi;
    const double lphi = dot(n, lfn);
    ll.kN += -depth * lphi;
    ldepth += -c.kN * lphi;
    ll.cN += ervn * lphi;
    a.erv = a.erv + n * (c.cN * lphi);
    ln = ln + in.erv * (c.cN * lphi);
    law_constants_vjp(m, mred, reff, ll, g);
    // geometry: depth = rs - d, n = delta / d, d = sqrt(d2), d2 = delta.delta
    ld -= ldepth;
    a.delta = a.delta + ln * (1.0 / d);
    ld -= dot(in.delta, ln) / (d * d);
    a.delta = a.delta + n * ld + in.delta * (2.0 * ld2);
    a.h[0] += lh0.x; a.h[1] += lh0.y; a.h[2] += lh0.z;
    a.h[3] += lh1.x; a.h[4] += lh1.y; a.h[5] += lh1.z;
    a.h[6] += lh2.x; a.h[7] += lh2.y; a.h[8] += lh2.z;
}

// ------------------------------------------------------------- wall law
// One particle and one planar wall: out = wall normal, depth = r - (p - o).out,
// endpoint velocity vel and world angular velocity om.
struct PWAdj {
    D3 p, vel, om;
    double h[9];
};
DEM_DEV void pw_law_vjp(const MatC& m, double dt, D3 out, double depth, double r, double mass, D3 vel, D3 om,
                        const double hin[9], D3 lF, D3 lC, const double lh_out[9], PWAdj& a, MatGrad& g)
{
    const D3 n = out * -1.0;
    const double lever = r - depth;
    const D3 rv = vel * -1.0;
    const double rvn = dot(rv, n);
    const D3 Z = cross(n, om);
    const D3 tv = rv - n * rvn + Z * lever;
    const D3 rw = om * -1.0;
    const double rwn = dot(rw, n);
    const D3 twr = n * rwn;
    const bool lev = fabs(lever) > 1.0e-30;
    const D3 Q = cross(n, tv);
    const D3 rlr = lev ? (rw - twr) + Q * (0.5 / lever) : rw - twr;
    const LawC<double> c = law_constants<double, MatC>(m, mass, r);
    const D3 fn = n * (-c.kN * depth) + n * (c.cN * rvn);
    const double fnn = norm(fn);
    const double flim = m.mu * fnn;
    const double ms = m.beta * r * fnn;
    const D3 h0 = mk(hin[0], hin[1], hin[2]), h1 = mk(hin[3], hin[4], hin[5]), h2 = mk(hin[6], hin[7], hin[8]);
    const D3 prev_t = transport_tangent(h1, n), prev_w = transport_axial(h2, n), prev_r = transport_tangent(h0, n);
    D3 st;
    const D3 fr = wall_response<double>(tv, c.kS, c.cS, dt, prev_t, flim, false, false, st);
    const double Lw = m.mu * m.muT * ms, Lr = m.muR * ms;

    D3 lfn = lF, lfr = lF, ln_unused = z3();
    double llever = 0.0, ldepth = 0.0;
    LawL ll = {0, 0, 0, 0, 0, 0, 0, 0};
    // couple = (tw + rl) + cross(n, fr) lever
    llever += dot(cross(n, fr), lC);
    cross_vjp(n, fr, lC * lever, ln_unused, lfr);
    D3 lrlr = z3(), lpr = z3();
    double lLr = 0.0;
    wall_response_vjp(rlr, c.kR, c.cR, dt, prev_r, Lr, true, true, lC, mk(lh_out[0], lh_out[1], lh_out[2]), lrlr, ll.kR,
                      ll.cR, lpr, lLr);
    D3 ltwr = z3(), lpw = z3();
    double lLw = 0.0;
    wall_response_vjp(twr, c.kT, c.cT, dt, prev_w, Lw, false, true, lC, mk(lh_out[6], lh_out[7], lh_out[8]), ltwr, ll.kT,
                      ll.cT, lpw, lLw);
    D3 ltv = z3(), lpt = z3();
    double lflim = 0.0;
    wall_response_vjp(tv, c.kS, c.cS, dt, prev_t, flim, false, false, lfr, mk(lh_out[3], lh_out[4], lh_out[5]), ltv,
                      ll.kS, ll.cS, lpt, lflim);
    const double lms = m.muR * lLr + m.mu * m.muT * lLw;
    g.muR += ms * lLr;
    g.mu += m.muT * ms * lLw + fnn * lflim;
    g.muT += m.mu * ms * lLw;
    norm_vjp(fn, m.beta * r * lms + m.mu * lflim, lfn);
    D3 lh0 = z3(), lh1 = z3(), lh2 = z3();
    transport_tangent_vjp(h0, n, lpr, lh0, ln_unused);
    transport_axial_vjp(h2, n, lpw, lh2, ln_unused);
    transport_tangent_vjp(h1, n, lpt, lh1, ln_unused);
    // rlr = rw - n (rw.n) [+ Q (0.5 / lever)], Q = n x tv
    D3 lrw = lrlr - n * dot(n, lrlr);
    if (lev) {
        const D3 lQ = lrlr * (0.5 / lever);
        llever += -dot(Q, lrlr) * 0.5 / (lever * lever);
        cross_vjp(n, tv, lQ, ln_unused, ltv);
    }
    lrw = lrw + n * dot(n, ltwr);
    a.om = a.om - lrw;
    // tv = rv - n (rv.n) + Z lever, Z = n x om
    D3 lrv = ltv - n * dot(n, ltv);
    llever += dot(Z, ltv);
    cross_vjp(n, om, ltv * lever, ln_unused, a.om);
    // fn = n (-kN depth) + n (cN rv.n)
    const double lphi = dot(n, lfn);
    ll.kN += -depth * lphi;
    ldepth += -c.kN * lphi;
    ll.cN += rvn * lphi;
    lrv = lrv + n * (c.cN * lphi);
    a.vel = a.vel - lrv;
    law_constants_vjp(m, mass, r, ll, g);
    // lever = r - depth; depth = r - (p - o).out
    ldepth -= llever;
    a.p = a.p - out * ldepth;
    a.h[0] += lh0.x; a.h[1] += lh0.y; a.h[2] += lh0.z;
    a.h[3] += lh1.x; a.h[4] += lh1.y; a.h[5] += lh1.z;
    a.h[6] += lh2.x; a.h[7] += lh2.y; a.h[8] += lh2.z;
}

}  // namespace demgb
