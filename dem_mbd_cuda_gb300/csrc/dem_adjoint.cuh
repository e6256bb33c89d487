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

#include <type_traits>

#include "dem_device.cuh"

namespace demgb {

using D3 = V3<double>;

// Adjoints of the material constants of one contact class: kN (kS = 2 kN / 7
// is folded in), mu, log(epsN) and log(epsS) (the denominators pi^2 + log^2
// are folded in), muT, muR.
template <typename R> struct MatGradT {
    R kN, mu, logN, logS, muT, muR;
};
using MatGrad = MatGradT<double>;

DEM_DEV D3 z3() { return mk(0.0, 0.0, 0.0); }
template <typename R> DEM_DEV V3<R> zr() { return mk<R>(R(0), R(0), R(0)); }

// ------------------------------------------------------------- primitives
// a x b: adjoint la += b x lo, lb += lo x a
template <typename R> DEM_DEV void cross_vjp(V3<R> a, V3<R> b, V3<R> lo, V3<R>& la, V3<R>& lb)
{
    la = la + cross(b, lo);
    lb = lb + cross(lo, a);
}
// |a|
template <typename R> DEM_DEV void norm_vjp(V3<R> a, R lo, V3<R>& la)
{
    const R n = norm(a);
    if (n > R(0)) la = la + a * (lo / n);
}
// The quaternion maps below take their inputs in R and add their adjoints
// into accumulators of type A: R = A = double is the FP64 reverse; R =
// float, A = double computes each increment in FP32 and adds it to the FP64
// adjoint that carries it from step to step (B: the accumulator of a
// second output, where it may differ).

// q / |q| (normalize_quat; the degenerate reset to identity has no adjoint)
template <typename R, typename A> DEM_DEV void normq_vjp(const R q[4], const R lo[4], A lq[4])
{
    const R n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (n2 <= R(1.0e-24)) return;
    const R inv = R(1.0) / sqrt(n2);
    R o[4], d = R(0.0);
    for (int k = 0; k < 4; ++k) { o[k] = q[k] * inv; d += o[k] * lo[k]; }
    for (int k = 0; k < 4; ++k) lq[k] += A((lo[k] - o[k] * d) * inv);
}
// quat_derivative G(q, w) = 0.5 q (x) (0, w)
template <typename R> DEM_DEV void quatd(const R q[4], V3<R> w, R o[4])
{
    o[0] = R(0.5) * (-q[1] * w.x - q[2] * w.y - q[3] * w.z);
    o[1] = R(0.5) * (q[0] * w.x + q[2] * w.z - q[3] * w.y);
    o[2] = R(0.5) * (q[0] * w.y - q[1] * w.z + q[3] * w.x);
    o[3] = R(0.5) * (q[0] * w.z + q[1] * w.y - q[2] * w.x);
}
template <typename R, typename A, typename B>
DEM_DEV void quatd_vjp(const R q[4], V3<R> w, const R lo[4], A lq[4], V3<B>& lw)
{
    lq[0] += A(R(0.5) * (lo[1] * w.x + lo[2] * w.y + lo[3] * w.z));
    lq[1] += A(R(0.5) * (-lo[0] * w.x - lo[2] * w.z + lo[3] * w.y));
    lq[2] += A(R(0.5) * (-lo[0] * w.y + lo[1] * w.z - lo[3] * w.x));
    lq[3] += A(R(0.5) * (-lo[0] * w.z - lo[1] * w.y + lo[2] * w.x));
    lw.x += B(R(0.5) * (-lo[0] * q[1] + lo[1] * q[0] + lo[2] * q[3] - lo[3] * q[2]));
    lw.y += B(R(0.5) * (-lo[0] * q[2] - lo[1] * q[3] + lo[2] * q[0] + lo[3] * q[1]));
    lw.z += B(R(0.5) * (-lo[0] * q[3] + lo[1] * q[2] - lo[2] * q[1] + lo[3] * q[0]));
}
// rot_iv(q, v) = R(q) v (body -> world)
template <typename R> DEM_DEV V3<R> rotq(const R q[4], V3<R> v)
{
    if constexpr (std::is_same<R, double>::value) {
        return rot_iv(q[0], q[1], q[2], q[3], v);
    } else {
        const R qw = q[0], qx = q[1], qy = q[2], qz = q[3];
        return {(R(1) - R(2) * (qy * qy + qz * qz)) * v.x + R(2) * (qx * qy - qw * qz) * v.y +
                    R(2) * (qx * qz + qw * qy) * v.z,
                R(2) * (qx * qy + qw * qz) * v.x + (R(1) - R(2) * (qx * qx + qz * qz)) * v.y +
                    R(2) * (qy * qz - qw * qx) * v.z,
                R(2) * (qx * qz - qw * qy) * v.x + R(2) * (qy * qz + qw * qx) * v.y +
                    (R(1) - R(2) * (qx * qx + qy * qy)) * v.z};
    }
}
template <typename R, typename A> DEM_DEV void rotq_vjp(const R q[4], V3<R> v, V3<R> lo, A lq[4], V3<A>& lv)
{
    const R qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    const R one = R(1.0), two = R(2.0), four = R(4.0);
    // lv += R^T lo
    lv.x += A((one - two * (qy * qy + qz * qz)) * lo.x + two * (qx * qy + qw * qz) * lo.y +
              two * (qx * qz - qw * qy) * lo.z);
    lv.y += A(two * (qx * qy - qw * qz) * lo.x + (one - two * (qx * qx + qz * qz)) * lo.y +
              two * (qy * qz + qw * qx) * lo.z);
    lv.z += A(two * (qx * qz + qw * qy) * lo.x + two * (qy * qz - qw * qx) * lo.y +
              (one - two * (qx * qx + qy * qy)) * lo.z);
    // lq += (d(R v)/dq)^T lo
    const R vx = v.x, vy = v.y, vz = v.z;
    lq[0] += A(lo.x * (-two * qz * vy + two * qy * vz) + lo.y * (two * qz * vx - two * qx * vz) +
               lo.z * (-two * qy * vx + two * qx * vy));
    lq[1] += A(lo.x * (two * qy * vy + two * qz * vz) + lo.y * (two * qy * vx - four * qx * vy - two * qw * vz) +
               lo.z * (two * qz * vx + two * qw * vy - four * qx * vz));
    lq[2] += A(lo.x * (-four * qy * vx + two * qx * vy + two * qw * vz) + lo.y * (two * qx * vx + two * qz * vz) +
               lo.z * (-two * qw * vx + two * qz * vy - four * qy * vz));
    lq[3] += A(lo.x * (-four * qz * vx - two * qw * vy + two * qx * vz) +
               lo.y * (two * qw * vx - four * qz * vy + two * qy * vz) + lo.z * (two * qx * vx + two * qy * vy));
}
// R(q)^T t (world -> body, the Euler-equation transform of the owner sum) is
// R(conj q) t
template <typename R> DEM_DEV V3<R> rotq_t(const R q[4], V3<R> t)
{
    const R c[4] = {q[0], -q[1], -q[2], -q[3]};
    return rotq(c, t);
}
template <typename R, typename A> DEM_DEV void rotq_t_vjp(const R q[4], V3<R> t, V3<R> lo, A lq[4], V3<A>& lt)
{
    const R c[4] = {q[0], -q[1], -q[2], -q[3]};
    A lc[4] = {A(0), A(0), A(0), A(0)};
    rotq_vjp(c, t, lo, lc, lt);
    lq[0] += lc[0]; lq[1] -= lc[1]; lq[2] -= lc[2]; lq[3] -= lc[3];
}

// --------------------------------------------------------- history maps
template <typename R> DEM_DEV void transport_tangent_vjp(V3<R> h, V3<R> n, V3<R> lo, V3<R>& lh, V3<R>& ln)
{
    const R pn = norm(h);
    const R hn = dot(h, n);
    const V3<R> proj = h - n * hn;
    const R qn = norm(proj);
    if (pn <= R(1.0e-30) || qn <= R(1.0e-30)) return;
    const R s = pn / qn;
    V3<R> lproj = lo * s;
    const R ls = dot(proj, lo);
    const R lpn = ls / qn, lqn = -ls * pn / (qn * qn);
    lproj = lproj + proj * (lqn / qn);
    lh = lh + h * (lpn / pn);
    const R nl = dot(n, lproj);
    lh = lh + (lproj - n * nl);
    ln = ln + lproj * (-hn) - h * nl;
}
template <typename R> DEM_DEV void transport_axial_vjp(V3<R> h, V3<R> n, V3<R> lo, V3<R>& lh, V3<R>& ln)
{
    const R pn = norm(h);
    if (pn <= R(1.0e-30)) return;
    const R al = dot(h, n);
    if (fabs(al) <= R(1.0e-30)) return;
    const R sg = al < R(0) ? R(-1) : R(1);
    ln = ln + lo * (sg * pn);
    lh = lh + h * (sg * dot(n, lo) / pn);
}

// limitedHistoryResponseRates (:267-299): (resp, stored) from (hrate,
// rrate, k, c, prev, limit); lr = adjoint of resp, ls = of stored.
template <typename R>
DEM_DEV void limited_rates_vjp(V3<R> hrate, V3<R> rrate, R k, R c, R dt, V3<R> prev, R limit, V3<R> lr, V3<R> ls,
                               V3<R>& lhrate, V3<R>& lrrate, R& lk, R& lc, V3<R>& lprev, R& llimit)
{
    const V3<R> delta = hrate * dt;
    const V3<R> inc = delta * k;
    const V3<R> et = inc + prev;
    const R tn = norm(et);
    V3<R> linc = zr<R>();
    if (tn > limit) {
        const V3<R> lR = lr + ls;
        if (norm(delta) > R(1.0e-14)) {
            const R g = limit / tn;
            V3<R> let = lR * g;
            const R lg = dot(et, lR);
            llimit += lg / tn;
            const R ltn = -lg * limit / (tn * tn);
            let = let + et * (ltn / tn);
            linc = let;
            lprev = lprev + let;
        } else {
            const R pn = norm(prev);
            if (pn > R(1.0e-14)) {
                const R g = limit / pn;
                lprev = lprev + lR * g;
                const R lg = dot(prev, lR);
                llimit += lg / pn;
                const R lpn = -lg * limit / (pn * pn);
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
template <typename R>
DEM_DEV void wall_response_vjp(V3<R> rate, R k, R c, R dt, V3<R> prev, R limit, bool check_damped, bool zero_at_zero,
                               V3<R> lr, V3<R> ls, V3<R>& lrate, R& lk, R& lc, V3<R>& lprev, R& llimit)
{
    const V3<R> delta = rate * dt;
    const V3<R> et = prev + delta * k;
    const V3<R> st = et + rate * c;
    const R tn = norm(check_damped ? st : et);
    V3<R> let = zr<R>();
    if (tn > limit) {
        const V3<R> lR = lr + ls;
        const R dn = norm(delta);
        if (dn > R(1.0e-14) && tn > R(1.0e-14)) {
            const V3<R> lt = check_damped ? st : et;
            const R g = limit / tn;
            V3<R> llt = lR * g;
            const R lg = dot(lt, lR);
            llimit += lg / tn;
            const R ltn = -lg * limit / (tn * tn);
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
template <typename R> struct LawLT {
    R kN, kS, cN, cS, kT, cT, kR, cR;
};
using LawL = LawLT<double>;
template <typename R, typename M>
DEM_DEV void law_constants_vjp(const M& m, R mred, R rterm, const LawLT<R>& l, MatGradT<R>& g)
{
    const R beta = R(m.beta), kN = R(m.kN), kS = R(m.kS), denN = R(m.denN), denS = R(m.denS);
    const R logN = R(m.logN), logS = R(m.logS);
    const R brs = beta * rterm * beta * rterm;
    R lkS = l.kS + R(2.0) * brs * l.kT;
    const R lcS = l.cS + R(2.0) * brs * l.cT;
    R lkN = l.kN + brs * l.kR;
    const R lcN = l.cN + brs * l.cR;
    // cN = -2 logN sqrt(kN mred / denN), denN = pi^2 + logN^2
    {
        const R A = kN * mred / denN, sA = sqrt(A);
        const R lA = -logN * lcN / sA;
        g.logN += R(-2.0) * sA * lcN;
        lkN += lA * mred / denN;
        const R lden = -lA * kN * mred / (denN * denN);
        g.logN += R(2.0) * logN * lden;
    }
    // cS = -2 logS sqrt(kS mred / denS)
    {
        const R A = kS * mred / denS, sA = sqrt(A);
        const R lA = -logS * lcS / sA;
        g.logS += R(-2.0) * sA * lcS;
        lkS += lA * mred / denS;
        const R lden = -lA * kS * mred / (denS * denS);
        g.logS += R(2.0) * logS * lden;
    }
    g.kN += lkN + lkS * R(2.0 / 7.0);
}

// --------------------------------------------------------- particle law
// Inputs of one contact side i (partner j): delta = p_j - p_i, radii,
// masses, endpoint and midpoint relative velocities (erv, mrv), world
// angular velocities (endpoint ew, midpoint mw), history h[9] before the
// step.  Output adjoints: force lF, couple lC (on i), stored history lh[9].
template <typename R> struct PPInT {
    V3<R> delta;
    R ri, rj, mi, mj;
    V3<R> erv, mrv, ewi, ewj, mwi, mwj;
    R h[9];
    R depth;  // the overlap, given by the caller of the FP32 form (from FP64 positions)
};
template <typename R> struct PPAdjT {
    V3<R> delta, erv, mrv, ewi, ewj, mwi, mwj;
    R h[9];
};
using PPIn = PPInT<double>;
using PPAdj = PPAdjT<double>;

// R = double: the FP64 form.  R = float: the same map in FP32 (material
// constants M = MatF); the overlap in.depth comes from the caller, who forms
// it from the FP64 positions (r_i + r_j - d cancels in FP32).
template <typename R, typename M>
DEM_DEV void pp_law_vjp(const M& m, R dt, const PPInT<R>& in, V3<R> lF, V3<R> lC, const R lh_out[9], PPAdjT<R>& a,
                        MatGradT<R>& g)
{
    const R mu = R(m.mu), muT = R(m.muT), muR = R(m.muR), beta = R(m.beta), coh = R(m.coh);
    // forward
    const R d2 = dot(in.delta, in.delta);
    const R d = sqrt(d2);
    const V3<R> n = in.delta * (R(1.0) / d);
    const R rs = in.ri + in.rj;
    R depth;
    if constexpr (std::is_same<R, double>::value) depth = rs - d;
    else depth = in.depth;
    const R mred = in.mi * in.mj / (in.mi + in.mj);
    const R reff = in.ri * in.rj / rs;
    const LawC<R> c = law_constants<R, M>(m, mred, reff);
    const R ervn = dot(in.erv, n);
    const R phi = -c.kN * depth + c.cN * ervn + coh * R(4.0) * c.brs;
    const V3<R> fn = n * phi;
    const R A = in.ri * in.ri - in.rj * in.rj;
    const R li = (A + d2) / (R(2.0) * d);
    const R lj = d - li;
    const V3<R> X1 = cross(n, in.ewi), X2 = cross(n, in.ewj), Y1 = cross(n, in.mwi), Y2 = cross(n, in.mwj);
    const R mrvn = dot(in.mrv, n);
    const V3<R> etv = in.erv - n * ervn + X1 * li + X2 * lj;
    const V3<R> mtv = in.mrv - n * mrvn + Y1 * li + Y2 * lj;
    const V3<R> h0 = mk(in.h[0], in.h[1], in.h[2]), h1 = mk(in.h[3], in.h[4], in.h[5]), h2 = mk(in.h[6], in.h[7], in.h[8]);
    const V3<R> prev_t = transport_tangent(h1, n);
    const R fnn = norm(fn);
    const R Lt = mu * fnn;
    V3<R> st;
    bool y;
    const V3<R> fr = limited_rates<R>(mtv, etv, c.kS, c.cS, dt, prev_t, Lt, st, y);
    const V3<R> erw = in.ewj - in.ewi, mrw = in.mwj - in.mwi;
    const R erwn = dot(erw, n), mrwn = dot(mrw, n);
    const V3<R> etw = n * erwn, mtw = n * mrwn;
    const V3<R> erl = erw - etw, mrl = mrw - mtw;
    const R ms = beta * reff * fnn;
    const V3<R> prev_w = transport_axial(h2, n);
    const R Lw = mu * muT * ms;
    const V3<R> prev_r = transport_tangent(h0, n);
    const R Lr = muR * ms;

    // reverse
    V3<R> ln = zr<R>(), lfn = lF, lfr = lF;
    R lli = 0, llj = 0, ld = 0, ld2 = 0, ldepth = 0;
    LawLT<R> ll = {0, 0, 0, 0, 0, 0, 0, 0};
    // couple = (tw + rl) + cross(n, fr) li
    const V3<R> lX = lC * li;
    lli += dot(cross(n, fr), lC);
    cross_vjp(n, fr, lX, ln, lfr);
    // roll channel
    V3<R> lmrl = zr<R>(), lerl = zr<R>(), lpr = zr<R>();
    R lLr = 0;
    limited_rates_vjp(mrl, erl, c.kR, c.cR, dt, prev_r, Lr, lC, mk(lh_out[0], lh_out[1], lh_out[2]), lmrl, lerl, ll.kR,
                      ll.cR, lpr, lLr);
    // twist channel
    V3<R> lmtw = zr<R>(), letw = zr<R>(), lpw = zr<R>();
    R lLw = 0;
    limited_rates_vjp(mtw, etw, c.kT, c.cT, dt, prev_w, Lw, lC, mk(lh_out[6], lh_out[7], lh_out[8]), lmtw, letw, ll.kT,
                      ll.cT, lpw, lLw);
    // tangential channel
    V3<R> lmtv = zr<R>(), letv = zr<R>(), lpt = zr<R>();
    R lLt = 0;
    limited_rates_vjp(mtv, etv, c.kS, c.cS, dt, prev_t, Lt, lfr, mk(lh_out[3], lh_out[4], lh_out[5]), lmtv, letv, ll.kS,
                      ll.cS, lpt, lLt);
    // limits
    R lms = muR * lLr + mu * muT * lLw;
    g.muR += ms * lLr;
    g.mu += muT * ms * lLw + fnn * lLt;
    g.muT += mu * ms * lLw;
    const R lfnn = beta * reff * lms + mu * lLt;
    norm_vjp(fn, lfnn, lfn);
    // transports
    V3<R> lh0 = zr<R>(), lh1 = zr<R>(), lh2 = zr<R>();
    transport_tangent_vjp(h0, n, lpr, lh0, ln);
    transport_axial_vjp(h2, n, lpw, lh2, ln);
    transport_tangent_vjp(h1, n, lpt, lh1, ln);
    // rolling and twisting rates: erl = erw - n (erw.n), etw = n (erw.n)
    V3<R> lerw = zr<R>(), lmrw = zr<R>();
    {
        const R nl = dot(n, lerl);
        lerw = lerw + lerl - n * nl;
        ln = ln + lerl * (-erwn) - erw * nl;
        const R nt = dot(n, letw);
        ln = ln + letw * erwn + erw * nt;
        lerw = lerw + n * nt;
    }
    {
        const R nl = dot(n, lmrl);
        lmrw = lmrw + lmrl - n * nl;
        ln = ln + lmrl * (-mrwn) - mrw * nl;
        const R nt = dot(n, lmtw);
        ln = ln + lmtw * mrwn + mrw * nt;
        lmrw = lmrw + n * nt;
    }
    a.ewj = a.ewj + lerw; a.ewi = a.ewi - lerw;
    a.mwj = a.mwj + lmrw; a.mwi = a.mwi - lmrw;
    // etv = erv - n (erv.n) + X1 li + X2 lj
    {
        const R nl = dot(n, letv);
        a.erv = a.erv + letv - n * nl;
        ln = ln + letv * (-ervn) - in.erv * nl;
        lli += dot(X1, letv);
        llj += dot(X2, letv);
        cross_vjp(n, in.ewi, letv * li, ln, a.ewi);
        cross_vjp(n, in.ewj, letv * lj, ln, a.ewj);
    }
    {
        const R nl = dot(n, lmtv);
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
    ld2 += lli / (R(2.0) * d);
    ld -= lli * (A + d2) / (R(2.0) * d * d);
    // fn = n phi
    ln = ln + lfn * phi;
    const R lphi = dot(n, lfn);
    ll.kN += -depth * lphi;
    ldepth += -c.kN * lphi;
    ll.cN += ervn * lphi;
    a.erv = a.erv + n * (c.cN * lphi);
    ln = ln + in.erv * (c.cN * lphi);
    law_constants_vjp(m, mred, reff, ll, g);
    // geometry: depth = rs - d, n = delta / d, d = sqrt(d2), d2 = delta.delta
    ld -= ldepth;
    a.delta = a.delta + ln * (R(1.0) / d);
    ld -= dot(in.delta, ln) / (d * d);
    a.delta = a.delta + n * ld + in.delta * (R(2.0) * ld2);
    a.h[0] += lh0.x; a.h[1] += lh0.y; a.h[2] += lh0.z;
    a.h[3] += lh1.x; a.h[4] += lh1.y; a.h[5] += lh1.z;
    a.h[6] += lh2.x; a.h[7] += lh2.y; a.h[8] += lh2.z;
}

// ------------------------------------------------------------- wall law
// One particle and one planar wall: out = wall normal, depth = r - (p - o).out,
// endpoint velocity vel and world angular velocity om.
template <typename R> struct PWAdjT {
    V3<R> p, vel, om;
    R h[9];
};
using PWAdj = PWAdjT<double>;
template <typename R, typename M>
DEM_DEV void pw_law_vjp(const M& m, R dt, V3<R> out, R depth, R r, R mass, V3<R> vel, V3<R> om, const R hin[9],
                        V3<R> lF, V3<R> lC, const R lh_out[9], PWAdjT<R>& a, MatGradT<R>& g)
{
    const R mu = R(m.mu), muT = R(m.muT), muR = R(m.muR), beta = R(m.beta);
    const V3<R> n = out * R(-1.0);
    const R lever = r - depth;
    const V3<R> rv = vel * R(-1.0);
    const R rvn = dot(rv, n);
    const V3<R> Z = cross(n, om);
    const V3<R> tv = rv - n * rvn + Z * lever;
    const V3<R> rw = om * R(-1.0);
    const R rwn = dot(rw, n);
    const V3<R> twr = n * rwn;
    const bool lev = fabs(lever) > R(1.0e-30);
    const V3<R> Q = cross(n, tv);
    const V3<R> rlr = lev ? (rw - twr) + Q * (R(0.5) / lever) : rw - twr;
    const LawC<R> c = law_constants<R, M>(m, mass, r);
    const V3<R> fn = n * (-c.kN * depth) + n * (c.cN * rvn);
    const R fnn = norm(fn);
    const R flim = mu * fnn;
    const R ms = beta * r * fnn;
    const V3<R> h0 = mk(hin[0], hin[1], hin[2]), h1 = mk(hin[3], hin[4], hin[5]), h2 = mk(hin[6], hin[7], hin[8]);
    const V3<R> prev_t = transport_tangent(h1, n), prev_w = transport_axial(h2, n), prev_r = transport_tangent(h0, n);
    V3<R> st;
    const V3<R> fr = wall_response<R>(tv, c.kS, c.cS, dt, prev_t, flim, false, false, st);
    const R Lw = mu * muT * ms, Lr = muR * ms;

    V3<R> lfn = lF, lfr = lF, ln_unused = zr<R>();
    R llever = 0, ldepth = 0;
    LawLT<R> ll = {0, 0, 0, 0, 0, 0, 0, 0};
    // couple = (tw + rl) + cross(n, fr) lever
    llever += dot(cross(n, fr), lC);
    cross_vjp(n, fr, lC * lever, ln_unused, lfr);
    V3<R> lrlr = zr<R>(), lpr = zr<R>();
    R lLr = 0;
    wall_response_vjp(rlr, c.kR, c.cR, dt, prev_r, Lr, true, true, lC, mk(lh_out[0], lh_out[1], lh_out[2]), lrlr, ll.kR,
                      ll.cR, lpr, lLr);
    V3<R> ltwr = zr<R>(), lpw = zr<R>();
    R lLw = 0;
    wall_response_vjp(twr, c.kT, c.cT, dt, prev_w, Lw, false, true, lC, mk(lh_out[6], lh_out[7], lh_out[8]), ltwr, ll.kT,
                      ll.cT, lpw, lLw);
    V3<R> ltv = zr<R>(), lpt = zr<R>();
    R lflim = 0;
    wall_response_vjp(tv, c.kS, c.cS, dt, prev_t, flim, false, false, lfr, mk(lh_out[3], lh_out[4], lh_out[5]), ltv,
                      ll.kS, ll.cS, lpt, lflim);
    const R lms = muR * lLr + mu * muT * lLw;
    g.muR += ms * lLr;
    g.mu += muT * ms * lLw + fnn * lflim;
    g.muT += mu * ms * lLw;
    norm_vjp(fn, beta * r * lms + mu * lflim, lfn);
    V3<R> lh0 = zr<R>(), lh1 = zr<R>(), lh2 = zr<R>();
    transport_tangent_vjp(h0, n, lpr, lh0, ln_unused);
    transport_axial_vjp(h2, n, lpw, lh2, ln_unused);
    transport_tangent_vjp(h1, n, lpt, lh1, ln_unused);
    // rlr = rw - n (rw.n) [+ Q (0.5 / lever)], Q = n x tv
    V3<R> lrw = lrlr - n * dot(n, lrlr);
    if (lev) {
        const V3<R> lQ = lrlr * (R(0.5) / lever);
        llever += -dot(Q, lrlr) * R(0.5) / (lever * lever);
        cross_vjp(n, tv, lQ, ln_unused, ltv);
    }
    lrw = lrw + n * dot(n, ltwr);
    a.om = a.om - lrw;
    // tv = rv - n (rv.n) + Z lever, Z = n x om
    V3<R> lrv = ltv - n * dot(n, ltv);
    llever += dot(Z, ltv);
    cross_vjp(n, om, ltv * lever, ln_unused, a.om);
    // fn = n (-kN depth) + n (cN rv.n)
    const R lphi = dot(n, lfn);
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

// ------------------------------------------- particle-triangle manifold
// The body contact of one component with one body (the loop of
// computeContactsKernel, src/cuda/cuda_contact_backend.cu:1148-1208, with
// advanceBodyManifoldHistory :855-949 and bodyContact :708-853), written
// once more in FP64 for the reverse sweep: the forward pieces below repeat
// what the PT kernels compute, and each has its vector-Jacobian product.
struct PTIn {
    D3 p, ev, mv, ew, mw;  // sphere: centre, endpoint and midpoint velocity, world spins (endpoint, midpoint)
    double rad, mass;
    D3 c, V, w;            // body: centre, velocity, body-frame spin
    double q[4];           // body orientation
    int ntri;
    const double* L[kPbTris];  // body-frame records of the manifold's triangles (15 values each)
    double h[9];           // the manifold's history before the step
};
struct PTOut {
    D3 pf, ptq, rf, bt;    // sphere force and couple, body force and torque
    double h[9];           // the history after the step
};
struct PTAdj {
    D3 p, ev, mv, ew, mw, c, V, w;
    double q[4];
    double h[9];
};

// circleEdgeArea with the cut parameters held fixed.  A cut lies on the
// circle, where the chord piece and the arc piece on either side of it agree,
// so moving it along the edge leaves the area unchanged: the derivative
// through the cuts is zero.
DEM_DEV void circle_edge_area_vjp(double ax, double ay, double bx, double by, double r, double lo, double& lax,
                                  double& lay, double& lbx, double& lby, double& lr)
{
    const double dx = bx - ax, dy = by - ay;
    const double aa = dx * dx + dy * dy;
    double cuts[4] = {0.0, 1.0, 0.0, 0.0};
    int n = 2;
    if (aa > 1.0e-30) {
        const double bb = 2.0 * (ax * dx + ay * dy);
        const double cc = (ax * ax + ay * ay) - r * r;
        const double disc = bb * bb - 4.0 * aa * cc;
        if (disc > 0.0) {
            const double root = sqrt(disc);
            const double t0 = (-bb - root) / (2.0 * aa);
            const double t1 = (-bb + root) / (2.0 * aa);
            if (t0 > 0.0 && t0 < 1.0) cuts[n++] = t0;
            if (t1 > 0.0 && t1 < 1.0) cuts[n++] = t1;
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            if (cuts[j] < cuts[i]) { const double tmp = cuts[i]; cuts[i] = cuts[j]; cuts[j] = tmp; }
    for (int i = 0; i + 1 < n; ++i) {
        const double ta = cuts[i], tb = cuts[i + 1];
        const double ux = ax + dx * ta, uy = ay + dy * ta;
        const double vx = ax + dx * tb, vy = ay + dy * tb;
        const double tm = 0.5 * (ta + tb);
        const double mx = ax + dx * tm, my = ay + dy * tm;
        const double cr = ux * vy - uy * vx;
        double lux, luy, lvx, lvy;
        if (mx * mx + my * my <= r * r) {
            const double lcr = 0.5 * lo;
            lux = lcr * vy; luy = -lcr * vx; lvx = -lcr * uy; lvy = lcr * ux;
        } else {
            const double dp = ux * vx + uy * vy;
            const double th = atan2(cr, dp);
            lr += r * th * lo;
            const double lth = 0.5 * r * r * lo, den = cr * cr + dp * dp;
            const double lcr = den > 0.0 ? lth * dp / den : 0.0, ldp = den > 0.0 ? -lth * cr / den : 0.0;
            lux = lcr * vy + ldp * vx; luy = -lcr * vx + ldp * vy;
            lvx = -lcr * uy + ldp * ux; lvy = lcr * ux + ldp * uy;
        }
        lax += lux * (1.0 - ta) + lvx * (1.0 - tb); lbx += lux * ta + lvx * tb;
        lay += luy * (1.0 - ta) + lvy * (1.0 - tb); lby += luy * ta + lvy * tb;
    }
}

// circleTriangleArea (:360-378)
DEM_DEV void circle_triangle_area_vjp(D3 normal, D3 ra, D3 rb, D3 rc, double r, double lo, D3& ln, D3& lra, D3& lrb,
                                      D3& lrc, double& lr)
{
    const D3 axis = fabs(normal.x) < 0.8 ? mk(1.0, 0.0, 0.0) : mk(0.0, 1.0, 0.0);
    const D3 w = cross(normal, axis);
    const double wl = norm(w);
    const D3 u = w * (1.0 / wl);
    const D3 v = cross(normal, u);
    const double ax = dot(ra, u), ay = dot(ra, v), bx = dot(rb, u), by = dot(rb, v), cx = dot(rc, u), cy = dot(rc, v);
    const double raw = circle_edge_area<double>(ax, ay, bx, by, r) + circle_edge_area<double>(bx, by, cx, cy, r) +
                       circle_edge_area<double>(cx, cy, ax, ay, r);
    if (fabs(raw) > kPi * r * r) {
        lr += 2.0 * kPi * r * lo;
        return;
    }
    const double l = raw < 0.0 ? -lo : lo;
    double lax = 0, lay = 0, lbx = 0, lby = 0, lcx = 0, lcy = 0;
    circle_edge_area_vjp(ax, ay, bx, by, r, l, lax, lay, lbx, lby, lr);
    circle_edge_area_vjp(bx, by, cx, cy, r, l, lbx, lby, lcx, lcy, lr);
    circle_edge_area_vjp(cx, cy, ax, ay, r, l, lcx, lcy, lax, lay, lr);
    lra = lra + u * lax + v * lay;
    lrb = lrb + u * lbx + v * lby;
    lrc = lrc + u * lcx + v * lcy;
    D3 lu = ra * lax + rb * lbx + rc * lcx;
    const D3 lv = ra * lay + rb * lby + rc * lcy;
    cross_vjp(normal, u, lv, ln, lu);
    const D3 lw = (lu - u * dot(u, lu)) * (1.0 / wl);
    D3 lax3 = z3();
    cross_vjp(normal, axis, lw, ln, lax3);
}

// tri_area_scale64: the adjoints of the scale (l_as) and of the distance
// (l_dist) to the world record (lW: v2..v4 and the normal) and the centre.
DEM_DEV void tri_area_scale_vjp(const double* W, D3 p, double r, double l_as, double l_dist, double* lW, D3& lp)
{
    const D3 n = mk(W[12], W[13], W[14]);
    const D3 a = mk(W[3], W[4], W[5]), b = mk(W[6], W[7], W[8]), c = mk(W[9], W[10], W[11]);
    const double dist = dot(n, p - a);
    const double c2 = r * r - dist * dist;
    const D3 ce = p - n * dist;
    const D3 ra = a - ce, rb = b - ce, rc = c - ce;
    const double rr = sqrt(c2);
    const double area = circle_triangle_area<double>(n, ra, rb, rc, rr);
    double l_area = 0.0, l_c2 = 0.0;
    if (area / (kPi * c2) < 1.0) {
        l_area = l_as / (kPi * c2);
        l_c2 = -l_as * area / (kPi * c2 * c2);
    }
    D3 ln = z3(), lra = z3(), lrb = z3(), lrc = z3();
    double lrr = 0.0;
    if (l_area != 0.0) circle_triangle_area_vjp(n, ra, rb, rc, rr, l_area, ln, lra, lrb, lrc, lrr);
    l_c2 += lrr / (2.0 * rr);
    const D3 lce = (lra + lrb + lrc) * -1.0;
    lp = lp + lce;
    ln = ln - lce * dist;
    double ldist = l_dist - dot(n, lce) - 2.0 * dist * l_c2;
    ln = ln + (p - a) * ldist;
    lp = lp + n * ldist;
    const D3 la = lra - n * ldist;
    lW[3] += la.x; lW[4] += la.y; lW[5] += la.z;
    lW[6] += lrb.x; lW[7] += lrb.y; lW[8] += lrb.z;
    lW[9] += lrc.x; lW[10] += lrc.y; lW[11] += lrc.z;
    lW[12] += ln.x; lW[13] += ln.y; lW[14] += ln.z;
}

// advanceBodyManifoldHistory: the manifold (normal mn, centre mc, distance
// md) updates the history h in place.
DEM_DEV void pt_history_fwd(const MatC& m, double dt, const PTIn& in, D3 wb, D3 mn, D3 mc, double md, double h[9])
{
    const D3 arm = mc - in.c;
    const D3 bvel = in.V + cross(wb, arm);
    const D3 erv = bvel - in.ev, mrv = bvel - in.mv;
    const D3 n = mn;
    const LawC<double> c = law_constants<double, MatC>(m, in.mass, in.rad);
    const double depth = in.rad - md;
    D3 fn = n * (-c.kN * depth) + n * (c.cN * dot(erv, n));
    fn = fn + n * (m.coh * 4.0 * c.brs);
    D3 tv = mrv - n * dot(mrv, n);
    tv = tv + cross(n, in.mw) * md;
    D3 st;
    bool y;
    limited_rates<double>(tv, tv, c.kS, c.cS, dt, transport_tangent(hload(h, 1), n), m.mu * norm(fn), st, y);
    hstore(h, 1, st);
    const D3 rw = wb - in.mw;
    const D3 twr = n * dot(rw, n);
    const D3 rlr = (rw - twr) + cross(n, tv) * (0.5 / fmax(md, 1.0e-14));
    const double ms = m.beta * in.rad * norm(fn);
    limited_rates<double>(twr, twr, c.kT, c.cT, dt, transport_axial(hload(h, 2), n), m.mu * m.muT * ms, st, y);
    hstore(h, 2, st);
    limited_rates<double>(rlr, rlr, c.kR, c.cR, dt, transport_tangent(hload(h, 0), n), m.muR * ms, st, y);
    hstore(h, 0, st);
}
// lh: adjoint of the history after the step (in).  Out: the adjoints of
// the manifold, of the sphere and body inputs and of the history before.
DEM_DEV void pt_history_vjp(const MatC& m, double dt, const PTIn& in, D3 wb, D3 mn, D3 mc, double md,
                            const double lh[9], D3& lmn, D3& lmc, double& lmd, D3& lwb, PTAdj& a, LawL& ll, MatGrad& g)
{
    const D3 arm = mc - in.c;
    const D3 bvel = in.V + cross(wb, arm);
    const D3 erv = bvel - in.ev, mrv = bvel - in.mv;
    const D3 n = mn;
    const LawC<double> c = law_constants<double, MatC>(m, in.mass, in.rad);
    const double depth = in.rad - md;
    const double ervn = dot(erv, n), mrvn = dot(mrv, n);
    const double phi = -c.kN * depth + c.cN * ervn + m.coh * 4.0 * c.brs;
    const D3 fn = n * phi;
    const double fnn = norm(fn);
    const D3 Y = cross(n, in.mw);
    const D3 tv = mrv - n * mrvn + Y * md;
    const D3 h0 = mk(in.h[0], in.h[1], in.h[2]), h1 = mk(in.h[3], in.h[4], in.h[5]), h2 = mk(in.h[6], in.h[7], in.h[8]);
    const D3 prev_t = transport_tangent(h1, n), prev_w = transport_axial(h2, n), prev_r = transport_tangent(h0, n);
    const D3 rw = wb - in.mw;
    const double rwn = dot(rw, n);
    const D3 twr = n * rwn;
    const double mdc = fmax(md, 1.0e-14), inv = 0.5 / mdc;
    const D3 Q = cross(n, tv);
    const D3 rlr = (rw - twr) + Q * inv;
    const double ms = m.beta * in.rad * fnn;
    const double Lt = m.mu * fnn, Lw = m.mu * m.muT * ms, Lr = m.muR * ms;
    D3 ln = z3();
    // roll (stored only)
    D3 lrlr = z3(), lrlr2 = z3(), lpr = z3();
    double lLr = 0.0;
    limited_rates_vjp(rlr, rlr, c.kR, c.cR, dt, prev_r, Lr, z3(), mk(lh[0], lh[1], lh[2]), lrlr, lrlr2, ll.kR, ll.cR,
                      lpr, lLr);
    lrlr = lrlr + lrlr2;
    // twist
    D3 ltwr = z3(), ltwr2 = z3(), lpw = z3();
    double lLw = 0.0;
    limited_rates_vjp(twr, twr, c.kT, c.cT, dt, prev_w, Lw, z3(), mk(lh[6], lh[7], lh[8]), ltwr, ltwr2, ll.kT, ll.cT,
                      lpw, lLw);
    ltwr = ltwr + ltwr2;
    // tangent
    D3 ltv = z3(), ltv2 = z3(), lpt = z3();
    double lLt = 0.0;
    limited_rates_vjp(tv, tv, c.kS, c.cS, dt, prev_t, Lt, z3(), mk(lh[3], lh[4], lh[5]), ltv, ltv2, ll.kS, ll.cS, lpt,
                      lLt);
    ltv = ltv + ltv2;
    // limits
    const double lms = m.muR * lLr + m.mu * m.muT * lLw;
    g.muR += ms * lLr;
    g.mu += m.muT * ms * lLw + fnn * lLt;
    g.muT += m.mu * ms * lLw;
    D3 lfn = z3();
    norm_vjp(fn, m.beta * in.rad * lms + m.mu * lLt, lfn);
    // transports of the history before the step
    D3 lh0 = z3(), lh1 = z3(), lh2 = z3();
    transport_tangent_vjp(h0, n, lpr, lh0, ln);
    transport_axial_vjp(h2, n, lpw, lh2, ln);
    transport_tangent_vjp(h1, n, lpt, lh1, ln);
    // rlr = (rw - twr) + Q inv, Q = n x tv
    D3 lrw = lrlr;
    ltwr = ltwr - lrlr;
    cross_vjp(n, tv, lrlr * inv, ln, ltv);
    if (md > 1.0e-14) lmd += -dot(Q, lrlr) * 0.5 / (md * md);
    // twr = n (rw.n)
    const double lrwn = dot(n, ltwr);
    ln = ln + ltwr * rwn + rw * lrwn;
    lrw = lrw + n * lrwn;
    // rw = wb - mw
    lwb = lwb + lrw;
    a.mw = a.mw - lrw;
    // tv = mrv - n (mrv.n) + Y md, Y = n x mw
    D3 lmrv = ltv;
    const double lmrvn = -dot(n, ltv);
    ln = ln - ltv * mrvn;
    lmd += dot(Y, ltv);
    cross_vjp(n, in.mw, ltv * md, ln, a.mw);
    lmrv = lmrv + n * lmrvn;
    ln = ln + mrv * lmrvn;
    // fn = n phi, phi = -kN depth + cN (erv.n) + coh 4 brs
    ln = ln + lfn * phi;
    const double lphi = dot(n, lfn);
    ll.kN += -depth * lphi;
    lmd += c.kN * lphi;  // depth = rad - md
    ll.cN += ervn * lphi;
    D3 lerv = n * (c.cN * lphi);
    ln = ln + erv * (c.cN * lphi);
    // erv = bvel - ev, mrv = bvel - mv, bvel = V + wb x arm, arm = mc - c
    const D3 lbvel = lerv + lmrv;
    a.ev = a.ev - lerv;
    a.mv = a.mv - lmrv;
    a.V = a.V + lbvel;
    D3 larm = z3();
    cross_vjp(wb, arm, lbvel, lwb, larm);
    lmc = lmc + larm;
    a.c = a.c - larm;
    lmn = lmn + ln;
    a.h[0] += lh0.x; a.h[1] += lh0.y; a.h[2] += lh0.z;
    a.h[3] += lh1.x; a.h[4] += lh1.y; a.h[5] += lh1.z;
    a.h[6] += lh2.x; a.h[7] += lh2.y; a.h[8] += lh2.z;
}

// bodyContact for one triangle with the history read only (dt = 0): sphere
// force pf and couple ptq, body force rf and torque bt (all scaled by the
// area share as).
DEM_DEV void pt_load_fwd(const MatC& m, const LawC<double>& c, const PTIn& in, D3 wb, const double* W, double as,
                         double dist, const double hn[9], D3& pf, D3& ptq, D3& rf, D3& bt)
{
    const D3 nout = mk(W[12], W[13], W[14]);
    const D3 ce = in.p - nout * dist;
    const D3 arm = ce - in.c;
    const D3 bvel = in.V + cross(wb, arm);
    const D3 n = nout * -1.0;
    const D3 rv = bvel - in.ev;
    const double depth = in.rad - dist;
    D3 fn = n * (-c.kN * depth) + n * (c.cN * dot(rv, n));
    fn = fn + n * (m.coh * 4.0 * c.brs);
    D3 tv = rv - n * dot(rv, n);
    tv = tv + cross(n, in.ew) * dist;
    D3 st;
    bool y;
    const D3 fr = limited_rates<double>(tv, tv, c.kS, c.cS, 0.0, transport_tangent(hload(hn, 1), n), m.mu * norm(fn),
                                        st, y);
    const D3 rw = wb - in.ew;
    const D3 twr = n * dot(rw, n);
    const D3 rlr = (rw - twr) + cross(n, tv) * (0.5 / fmax(dist, 1.0e-14));
    const double ms = m.beta * in.rad * norm(fn);
    const D3 tw = limited_rates<double>(twr, twr, c.kT, c.cT, 0.0, transport_axial(hload(hn, 2), n), m.mu * m.muT * ms,
                                        st, y);
    const D3 rl = limited_rates<double>(rlr, rlr, c.kR, c.cR, 0.0, transport_tangent(hload(hn, 0), n), m.muR * ms, st, y);
    const D3 F = fn + fr, cm = tw + rl;
    pf = F * as;
    ptq = (cm + cross(n, fr) * dist) * as;
    rf = F * (-as);
    bt = cross(arm, F) * (-as) + cm * (-as);
}
DEM_DEV void pt_load_vjp(const MatC& m, const LawC<double>& c, const PTIn& in, D3 wb, const double* W, double as,
                         double dist, const double hn[9], D3 lpf, D3 lptq, D3 lrf, D3 lbt, double& l_as, double& l_dist,
                         double* lW, D3& lwb, double lhn[9], PTAdj& a, LawL& ll, MatGrad& g)
{
    const D3 nout = mk(W[12], W[13], W[14]);
    const D3 ce = in.p - nout * dist;
    const D3 arm = ce - in.c;
    const D3 bvel = in.V + cross(wb, arm);
    const D3 n = nout * -1.0;
    const D3 rv = bvel - in.ev;
    const double depth = in.rad - dist;
    const double rvn = dot(rv, n);
    const double phi = -c.kN * depth + c.cN * rvn + m.coh * 4.0 * c.brs;
    const D3 fn = n * phi;
    const double fnn = norm(fn);
    const D3 Z = cross(n, in.ew);
    const D3 tv = rv - n * rvn + Z * dist;
    const D3 h0 = hload(hn, 0), h1 = hload(hn, 1), h2 = hload(hn, 2);
    const D3 prev_t = transport_tangent(h1, n), prev_w = transport_axial(h2, n), prev_r = transport_tangent(h0, n);
    D3 st;
    bool y;
    const double Lt = m.mu * fnn;
    const D3 fr = limited_rates<double>(tv, tv, c.kS, c.cS, 0.0, prev_t, Lt, st, y);
    const D3 rw = wb - in.ew;
    const double rwn = dot(rw, n);
    const D3 twr = n * rwn;
    const double inv = 0.5 / fmax(dist, 1.0e-14);
    const D3 Q = cross(n, tv);
    const D3 rlr = (rw - twr) + Q * inv;
    const double ms = m.beta * in.rad * fnn;
    const double Lw = m.mu * m.muT * ms, Lr = m.muR * ms;
    const D3 tw = limited_rates<double>(twr, twr, c.kT, c.cT, 0.0, prev_w, Lw, st, y);
    const D3 rl = limited_rates<double>(rlr, rlr, c.kR, c.cR, 0.0, prev_r, Lr, st, y);
    const D3 F = fn + fr, cm = tw + rl;
    const D3 nfr = cross(n, fr);
    const D3 armF = cross(arm, F);
    // outputs: pf = F as, ptq = (cm + nfr dist) as, rf = -F as, bt = -(armF + cm) as
    D3 lF = lpf * as - lrf * as;
    D3 lcm = lptq * as - lbt * as;
    l_as += dot(F, lpf) + dot(cm + nfr * dist, lptq) - dot(F, lrf) - dot(armF + cm, lbt);
    D3 ln = z3(), lfr = z3(), larm = z3();
    cross_vjp(n, fr, lptq * (as * dist), ln, lfr);
    l_dist += dot(nfr, lptq) * as;
    cross_vjp(arm, F, lbt * (-as), larm, lF);
    D3 lfn = lF;
    lfr = lfr + lF;
    // roll and twist responses
    D3 lrlr = z3(), lrlr2 = z3(), lpr = z3();
    double lLr = 0.0;
    limited_rates_vjp(rlr, rlr, c.kR, c.cR, 0.0, prev_r, Lr, lcm, z3(), lrlr, lrlr2, ll.kR, ll.cR, lpr, lLr);
    lrlr = lrlr + lrlr2;
    D3 ltwr = z3(), ltwr2 = z3(), lpw = z3();
    double lLw = 0.0;
    limited_rates_vjp(twr, twr, c.kT, c.cT, 0.0, prev_w, Lw, lcm, z3(), ltwr, ltwr2, ll.kT, ll.cT, lpw, lLw);
    ltwr = ltwr + ltwr2;
    // tangential response
    D3 ltv = z3(), ltv2 = z3(), lpt = z3();
    double lLt = 0.0;
    limited_rates_vjp(tv, tv, c.kS, c.cS, 0.0, prev_t, Lt, lfr, z3(), ltv, ltv2, ll.kS, ll.cS, lpt, lLt);
    ltv = ltv + ltv2;
    const double lms = m.muR * lLr + m.mu * m.muT * lLw;
    g.muR += ms * lLr;
    g.mu += m.muT * ms * lLw + fnn * lLt;
    g.muT += m.mu * ms * lLw;
    norm_vjp(fn, m.beta * in.rad * lms + m.mu * lLt, lfn);
    D3 lh0 = z3(), lh1 = z3(), lh2 = z3();
    transport_tangent_vjp(h0, n, lpr, lh0, ln);
    transport_axial_vjp(h2, n, lpw, lh2, ln);
    transport_tangent_vjp(h1, n, lpt, lh1, ln);
    lhn[0] += lh0.x; lhn[1] += lh0.y; lhn[2] += lh0.z;
    lhn[3] += lh1.x; lhn[4] += lh1.y; lhn[5] += lh1.z;
    lhn[6] += lh2.x; lhn[7] += lh2.y; lhn[8] += lh2.z;
    // rlr = (rw - twr) + Q inv, Q = n x tv
    D3 lrw = lrlr;
    ltwr = ltwr - lrlr;
    cross_vjp(n, tv, lrlr * inv, ln, ltv);
    if (dist > 1.0e-14) l_dist += -dot(Q, lrlr) * 0.5 / (dist * dist);
    const double lrwn = dot(n, ltwr);
    ln = ln + ltwr * rwn + rw * lrwn;
    lrw = lrw + n * lrwn;
    lwb = lwb + lrw;
    a.ew = a.ew - lrw;
    // tv = rv - n rvn + Z dist, Z = n x ew
    D3 lrv = ltv;
    double lrvn = -dot(n, ltv);
    ln = ln - ltv * rvn;
    l_dist += dot(Z, ltv);
    cross_vjp(n, in.ew, ltv * dist, ln, a.ew);
    // fn = n phi
    ln = ln + lfn * phi;
    const double lphi = dot(n, lfn);
    ll.kN += -depth * lphi;
    l_dist += c.kN * lphi;  // depth = rad - dist
    ll.cN += rvn * lphi;
    lrvn += c.cN * lphi;
    lrv = lrv + n * lrvn;
    ln = ln + rv * lrvn;
    // rv = bvel - ev, bvel = V + wb x arm, arm = ce - c, ce = p - nout dist, n = -nout
    a.ev = a.ev - lrv;
    a.V = a.V + lrv;
    cross_vjp(wb, arm, lrv, lwb, larm);
    a.c = a.c - larm;
    a.p = a.p + larm;
    const D3 lnout = larm * (-dist) - ln;
    l_dist += -dot(nout, larm);
    lW[12] += lnout.x; lW[13] += lnout.y; lW[14] += lnout.z;
}

// The whole manifold: triangle records, area shares, manifold, history
// update and the loads of each triangle.  Returns false without a manifold
// (no triangle with a share).
DEM_DEV bool pt_manifold_fwd(const MatC& m, double dt, const PTIn& in, PTOut& o)
{
    const D3 wb = rotq(in.q, in.w);
    double W[kPbTris][16], as[kPbTris], dist[kPbTris];
    double tot = 0.0, wd = 0.0;
    D3 wn = z3(), wc = z3();
    for (int t = 0; t < in.ntri; ++t) {
        double gc[3];
        tri_world(in.L[t], in.q[0], in.q[1], in.q[2], in.q[3], in.c.x, in.c.y, in.c.z, W[t], gc);
        as[t] = tri_area_scale64(W[t], in.p, in.rad, dist[t]);
        if (as[t] <= 0.0) continue;
        const D3 out = mk(W[t][12], W[t][13], W[t][14]);
        tot += as[t];
        wn = wn + out * (-as[t]);
        wc = wc + (in.p - out * dist[t]) * as[t];
        wd += dist[t] * as[t];
    }
    o.pf = o.ptq = o.rf = o.bt = z3();
    for (int k = 0; k < 9; ++k) o.h[k] = in.h[k];
    if (tot <= 0.0) return false;
    const D3 mn = normalized(wn), mc = wc * (1.0 / tot);
    const double md = wd / tot;
    pt_history_fwd(m, dt, in, wb, mn, mc, md, o.h);
    const LawC<double> lc = law_constants<double, MatC>(m, in.mass, in.rad);
    for (int t = 0; t < in.ntri; ++t) {
        if (as[t] <= 0.0 || dist[t] <= 0.0 || in.rad - dist[t] <= 0.0) continue;
        D3 pf, ptq, rf, bt;
        pt_load_fwd(m, lc, in, wb, W[t], as[t], dist[t], o.h, pf, ptq, rf, bt);
        o.pf = o.pf + pf; o.ptq = o.ptq + ptq; o.rf = o.rf + rf; o.bt = o.bt + bt;
    }
    return true;
}
// Adjoints of the sums (lpf, lptq, lrf, lbt) and of the history after the
// step (lh) to the inputs (a, added) and the materials (g, added).
DEM_DEV void pt_manifold_vjp(const MatC& m, double dt, const PTIn& in, D3 lpf, D3 lptq, D3 lrf, D3 lbt,
                             const double lh[9], PTAdj& a, MatGrad& g)
{
    const D3 wb = rotq(in.q, in.w);
    double W[kPbTris][16], as[kPbTris], dist[kPbTris];
    double tot = 0.0, wd = 0.0;
    D3 wn = z3(), wc = z3();
    for (int t = 0; t < in.ntri; ++t) {
        double gc[3];
        tri_world(in.L[t], in.q[0], in.q[1], in.q[2], in.q[3], in.c.x, in.c.y, in.c.z, W[t], gc);
        as[t] = tri_area_scale64(W[t], in.p, in.rad, dist[t]);
        if (as[t] <= 0.0) continue;
        const D3 out = mk(W[t][12], W[t][13], W[t][14]);
        tot += as[t];
        wn = wn + out * (-as[t]);
        wc = wc + (in.p - out * dist[t]) * as[t];
        wd += dist[t] * as[t];
    }
    if (tot <= 0.0) return;
    const double wnl = norm(wn);
    const D3 mn = wn * (1.0 / wnl), mc = wc * (1.0 / tot);
    const double md = wd / tot;
    double hn[9];
    for (int k = 0; k < 9; ++k) hn[k] = in.h[k];
    pt_history_fwd(m, dt, in, wb, mn, mc, md, hn);
    const LawC<double> lc = law_constants<double, MatC>(m, in.mass, in.rad);
    LawL ll = {0, 0, 0, 0, 0, 0, 0, 0};
    double las[kPbTris], ldist[kPbTris], lW[kPbTris][16];
    for (int t = 0; t < in.ntri; ++t) {
        las[t] = ldist[t] = 0.0;
        for (int k = 0; k < 16; ++k) lW[t][k] = 0.0;
    }
    D3 lwb = z3();
    double lhn[9];
    for (int k = 0; k < 9; ++k) lhn[k] = lh[k];
    // the loads, with the updated history read only
    for (int t = 0; t < in.ntri; ++t) {
        if (as[t] <= 0.0 || dist[t] <= 0.0 || in.rad - dist[t] <= 0.0) continue;
        pt_load_vjp(m, lc, in, wb, W[t], as[t], dist[t], hn, lpf, lptq, lrf, lbt, las[t], ldist[t], lW[t], lwb, lhn, a,
                    ll, g);
    }
    // the history update
    D3 lmn = z3(), lmc = z3();
    double lmd = 0.0;
    pt_history_vjp(m, dt, in, wb, mn, mc, md, lhn, lmn, lmc, lmd, lwb, a, ll, g);
    law_constants_vjp(m, in.mass, in.rad, ll, g);
    // the manifold: mn = wn / |wn|, mc = wc / tot, md = wd / tot
    const D3 lwn = (lmn - mn * dot(mn, lmn)) * (1.0 / wnl);
    const D3 lwc = lmc * (1.0 / tot);
    const double ltot = -dot(lmc, mc) / tot - lmd * md / tot, lwd = lmd / tot;
    for (int t = 0; t < in.ntri; ++t) {
        if (as[t] <= 0.0) continue;
        const D3 out = mk(W[t][12], W[t][13], W[t][14]);
        const D3 ce = in.p - out * dist[t];
        las[t] += ltot - dot(lwn, out) + dot(lwc, ce) + lwd * dist[t];
        const D3 lce = lwc * as[t];
        const D3 lout = lwn * (-as[t]) - lce * dist[t];
        ldist[t] += -dot(out, lce) + lwd * as[t];
        a.p = a.p + lce;
        lW[t][12] += lout.x; lW[t][13] += lout.y; lW[t][14] += lout.z;
        tri_area_scale_vjp(W[t], in.p, in.rad, las[t], ldist[t], lW[t], a.p);
        // the record: W_k = R(q) L_k + c (v2..v4), W_n = R(q) L_n
        for (int k = 1; k < 4; ++k) {
            const D3 lv = mk(lW[t][3 * k], lW[t][3 * k + 1], lW[t][3 * k + 2]);
            a.c = a.c + lv;
            D3 lunused = z3();
            rotq_vjp(in.q, mk(in.L[t][3 * k], in.L[t][3 * k + 1], in.L[t][3 * k + 2]), lv, a.q, lunused);
        }
        D3 lunused = z3();
        rotq_vjp(in.q, mk(in.L[t][12], in.L[t][13], in.L[t][14]), mk(lW[t][12], lW[t][13], lW[t][14]), a.q, lunused);
    }
    // wb = R(q) w
    rotq_vjp(in.q, in.w, lwb, a.q, a.w);
}

// ------------------------------------------------------------ body leapfrog
// The host MBD step of a dynamic body (DynEqnBodySet, src/dyneq.cpp:97-130,
// and the body leapfrog, src/cuda_simulation_integrator.cpp:348-374,
// 401-425).  A record of one step holds the pose the force evaluation used,
// the loads and the state after the half update; the adjoint fields follow.
constexpr int kBrC = 0, kBrQ = 3, kBrV = 7, kBrW = 10, kBrF = 13, kBrHV = 19, kBrHW = 22, kBrHQ = 25, kBrHDQ = 29,
              kBrAcc = 33, kBrDom = 36, kBR = 39;
constexpr int kBlC = 0, kBlQ = 3, kBlV = 7, kBlW = 10, kBlHV = 13, kBlHW = 16, kBlHDQ = 19, kBlAcc = 23, kBlDom = 26,
              kBlF = 29, kBL = 35;

DEM_DEV D3 ldv3(const double* a, int f) { return mk(a[f], a[f + 1], a[f + 2]); }
DEM_DEV void stv3(double* a, int f, D3 v) { a[f] = v.x; a[f + 1] = v.y; a[f + 2] = v.z; }

// acc = F / m; dom = (M(q) T - gyroscopic(W)) / I, M = Quat2DCM (the
// squared form of src/matrixtrans.cpp:36-63), I the principal inertia.
DEM_DEV void body_dyn(const double* F, const double q[4], D3 W, const double bc[4], D3& acc, D3& dom)
{
    const double m = bc[0], I0 = bc[1], I4 = bc[2], I8 = bc[3];
    acc = mk(F[0] / m, F[1] / m, F[2] / m);
    const double qq[10] = {q[0] * q[0], q[1] * q[1], q[2] * q[2], q[3] * q[3], 2.0 * q[0] * q[1], 2.0 * q[0] * q[2],
                           2.0 * q[0] * q[3], 2.0 * q[1] * q[2], 2.0 * q[1] * q[3], 2.0 * q[2] * q[3]};
    const double M[9] = {qq[0] + qq[1] - qq[2] - qq[3], qq[7] + qq[6], qq[8] - qq[5],
                         qq[7] - qq[6], qq[0] - qq[1] + qq[2] - qq[3], qq[9] + qq[4],
                         qq[8] + qq[5], qq[9] - qq[4], qq[0] - qq[1] - qq[2] + qq[3]};
    const double t0 = M[0] * F[3] + M[1] * F[4] + M[2] * F[5];
    const double t1 = M[3] * F[3] + M[4] * F[4] + M[5] * F[5];
    const double t2 = M[6] * F[3] + M[7] * F[4] + M[8] * F[5];
    dom = mk((t0 - (I8 - I4) * W.z * W.y) / I0, (t1 - (I0 - I8) * W.x * W.z) / I4, (t2 - (I4 - I0) * W.y * W.x) / I8);
}
DEM_DEV void body_dyn_vjp(const double* F, const double q[4], D3 W, const double bc[4], D3 lacc, D3 ldom, double* lF,
                          double lq[4], D3& lW)
{
    const double m = bc[0], I0 = bc[1], I4 = bc[2], I8 = bc[3];
    lF[0] += lacc.x / m; lF[1] += lacc.y / m; lF[2] += lacc.z / m;
    const double lt[3] = {ldom.x / I0, ldom.y / I4, ldom.z / I8};
    const double qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    const double M[9] = {qw * qw + qx * qx - qy * qy - qz * qz, 2.0 * qx * qy + 2.0 * qw * qz, 2.0 * qx * qz - 2.0 * qw * qy,
                         2.0 * qx * qy - 2.0 * qw * qz, qw * qw - qx * qx + qy * qy - qz * qz, 2.0 * qy * qz + 2.0 * qw * qx,
                         2.0 * qx * qz + 2.0 * qw * qy, 2.0 * qy * qz - 2.0 * qw * qx, qw * qw - qx * qx - qy * qy + qz * qz};
    // dM_rc / dq (rows of M, each a gradient in (qw, qx, qy, qz))
    const double dM[9][4] = {{2 * qw, 2 * qx, -2 * qy, -2 * qz}, {2 * qz, 2 * qy, 2 * qx, 2 * qw},
                             {-2 * qy, 2 * qz, -2 * qw, 2 * qx}, {-2 * qz, 2 * qy, 2 * qx, -2 * qw},
                             {2 * qw, -2 * qx, 2 * qy, -2 * qz}, {2 * qx, 2 * qw, 2 * qz, 2 * qy},
                             {2 * qy, 2 * qz, 2 * qw, 2 * qx}, {-2 * qx, -2 * qw, 2 * qz, 2 * qy},
                             {2 * qw, -2 * qx, -2 * qy, 2 * qz}};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            lF[3 + c] += M[3 * r + c] * lt[r];
            const double lM = lt[r] * F[3 + c];
            for (int k = 0; k < 4; ++k) lq[k] += lM * dM[3 * r + c][k];
        }
    lW.z += -lt[0] * (I8 - I4) * W.y; lW.y += -lt[0] * (I8 - I4) * W.z;
    lW.x += -lt[1] * (I0 - I8) * W.z; lW.z += -lt[1] * (I0 - I8) * W.x;
    lW.y += -lt[2] * (I4 - I0) * W.x; lW.x += -lt[2] * (I4 - I0) * W.y;
}
// Reverse of the half update of one step (record rec; first: the start's
// half step).  Lb holds the adjoints of the state after it (hv, hw carried,
// hdq, acc, dom) and of the pose; on return it holds the adjoint of the
// loads (kBlF) and the pose adjoint gains the update's terms.
DEM_DEV void body_half_vjp(const double* rec, const double bc[4], double dt, bool first, double* Lb)
{
    const double half = 0.5 * dt;
    const double* q = rec + kBrQ;
    const D3 W = ldv3(rec, kBrW);
    const double* hq = rec + kBrHQ;
    const D3 hw = ldv3(rec, kBrHW);
    double lhq[4] = {0, 0, 0, 0};
    D3 lhw = ldv3(Lb, kBlHW);
    quatd_vjp(hq, hw, Lb + kBlHDQ, lhq, lhw);
    double g[4], r[4], lr[4] = {0, 0, 0, 0};
    quatd(q, W, g);
    for (int k = 0; k < 4; ++k) r[k] = q[k] + g[k] * half;
    normq_vjp(r, lhq, lr);
    double* lq = Lb + kBlQ;
    for (int k = 0; k < 4; ++k) lq[k] += lr[k];
    double lg[4];
    for (int k = 0; k < 4; ++k) lg[k] = lr[k] * half;
    D3 lW = ldv3(Lb, kBlW);
    quatd_vjp(q, W, lg, lq, lW);
    const D3 lhv = ldv3(Lb, kBlHV);
    const double f = first ? half : dt;
    const D3 lacc = ldv3(Lb, kBlAcc) + lhv * f, ldom = ldv3(Lb, kBlDom) + lhw * f;
    if (first) {
        stv3(Lb, kBlV, ldv3(Lb, kBlV) + lhv);
        lW = lW + lhw;
        stv3(Lb, kBlHV, z3());
        stv3(Lb, kBlHW, z3());
    } else {
        stv3(Lb, kBlHW, lhw);
    }
    double lF[6] = {0, 0, 0, 0, 0, 0};
    body_dyn_vjp(rec + kBrF, q, W, bc, lacc, ldom, lF, lq, lW);
    stv3(Lb, kBlW, lW);
    for (int k = 0; k < 6; ++k) Lb[kBlF + k] = lF[k];
    stv3(Lb, kBlAcc, z3());
    stv3(Lb, kBlDom, z3());
    for (int k = 0; k < 4; ++k) Lb[kBlHDQ + k] = 0.0;
}
// Reverse of the position update into a step from the previous one's record.
DEM_DEV void body_pos_vjp(const double* prev, double dt, double* Lb)
{
    const double half = 0.5 * dt;
    const D3 lc = ldv3(Lb, kBlC), lV = ldv3(Lb, kBlV), lW = ldv3(Lb, kBlW);
    stv3(Lb, kBlHV, ldv3(Lb, kBlHV) + lc * dt + lV);
    stv3(Lb, kBlAcc, lV * half);
    stv3(Lb, kBlHW, ldv3(Lb, kBlHW) + lW);
    stv3(Lb, kBlDom, lW * half);
    double r[4], lr[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k) r[k] = prev[kBrQ + k] + prev[kBrHDQ + k] * dt;
    normq_vjp(r, Lb + kBlQ, lr);
    for (int k = 0; k < 4; ++k) {
        Lb[kBlQ + k] = lr[k];
        Lb[kBlHDQ + k] = lr[k] * dt;
    }
    stv3(Lb, kBlV, z3());
    stv3(Lb, kBlW, z3());
}

}  // namespace demgb
