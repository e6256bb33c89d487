// The particle-triangle candidate filter against the area routine, on the
// host.  tri_disk (dem_device.cuh) rejects a triangle without the edge sum
// when the contact disk lies beyond one of its edge lines (or out of reach
// of its circumradius); the engine then takes the scale as 0.  That is
// exact only if the reference's edge sum (circle_triangle_area, the
// restatement of circleTriangleArea) gives a scale at or below its 1e-12
// threshold for every rejected triangle.  Random disks placed just beyond an
// edge, beside a vertex, far away and across the triangle, on triangles of
// every shape and size ratio: for each rejected one the area scale must be
// below the threshold, and the filter must keep every triangle whose scale
// is above it.  Prints "ALL OK" when every case passes.
#include <cmath>
#include <cstdio>
#include <random>

#include "../dem_mbd_cuda_gb300/csrc/dem_device.cuh"

using namespace demgb;

static std::mt19937_64 rng(20261204);
static double U(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }

int main()
{
    long rejected = 0, by_edge = 0, kept = 0, bad = 0, missed = 0;
    for (int trial = 0; trial < 400000; ++trial) {
        // a triangle in a random plane, edges 1e-3 to 3e-2 m, anywhere in a
        // metre-sized box
        const V3<double> o = mk(U(-0.5, 0.5), U(-0.5, 0.5), U(-0.5, 0.5));
        V3<double> n = mk(U(-1, 1), U(-1, 1), U(-1, 1));
        n = n * (1.0 / norm(n));
        const V3<double> ax = fabs(n.x) < 0.8 ? mk(1.0, 0.0, 0.0) : mk(0.0, 1.0, 0.0);
        V3<double> u = cross(n, ax);
        u = u * (1.0 / norm(u));
        const V3<double> v = cross(n, u);
        const double scale = std::exp(U(std::log(1e-3), std::log(3e-2)));
        double P[3][2];
        for (auto& q : P) { q[0] = U(-1, 1) * scale; q[1] = U(-1, 1) * scale; }
        double W[16];
        for (int k = 0; k < 3; ++k) {
            const V3<double> p = o + u * P[k][0] + v * P[k][1];
            W[3 + 3 * k] = p.x; W[4 + 3 * k] = p.y; W[5 + 3 * k] = p.z;
        }
        // the triangle's normal (either side) and its circumradius about the
        // centroid, as the world record holds them
        const V3<double> a = mk(W[3], W[4], W[5]), b = mk(W[6], W[7], W[8]), c = mk(W[9], W[10], W[11]);
        V3<double> tn = cross(b - a, c - a);
        if (norm(tn) < 1e-12) continue;
        tn = tn * (1.0 / norm(tn));
        W[12] = tn.x; W[13] = tn.y; W[14] = tn.z;
        const V3<double> g = (a + b + c) * (1.0 / 3.0);
        W[15] = std::sqrt(std::fmax(dot(a - g, a - g), std::fmax(dot(b - g, b - g), dot(c - g, c - g)))) *
                    (1.0 + 1e-12) + 1e-15;
        W[0] = W[1] = W[2] = 0.0;
        // a sphere above the plane: its disk centre near an edge, a vertex or
        // anywhere around, radius 1e-4 to 2e-3 m, overlap up to its radius
        const double r = std::exp(U(std::log(1e-4), std::log(2e-3)));
        const double dist = U(1e-9, 1.0) * r;
        const double rc = std::sqrt(r * r - dist * dist);
        V3<double> ce;
        const int kind = trial % 4;
        const int e = trial % 3;
        const V3<double> pa = e == 0 ? a : e == 1 ? b : c, pb = e == 0 ? b : e == 1 ? c : a;
        const V3<double> other = e == 0 ? c : e == 1 ? a : b;
        if (kind == 0) {
            // beyond edge (pa, pb) by about the disk radius
            const V3<double> m = pa + (pb - pa) * U(-0.2, 1.2);
            V3<double> away = cross(pb - pa, tn);
            if (dot(away, other - pa) > 0) away = away * -1.0;
            away = away * (1.0 / norm(away));
            ce = m + away * (rc * U(0.999, 1.01));
        } else if (kind == 1) {
            ce = pa + (u * U(-1, 1) + v * U(-1, 1)) * rc * 1.2;
        } else if (kind == 2) {
            ce = g + (u * U(-1, 1) + v * U(-1, 1)) * (scale * 3.0);
        } else {
            ce = g + (u * U(-1, 1) + v * U(-1, 1)) * (scale + rc);
        }
        const V3<double> p = ce + tn * dist;
        TriDisk d;
        const bool meet = tri_disk(W, p, r, d);
        double dist64;
        const double sc = tri_area_scale64(W, p, r, dist64);
        // the reference's scale with no shortcut: the edge sum itself
        double ref = 0.0;
        {
            const double dd = dot(tn, p - a);
            const double c2 = r * r - dd * dd;
            if (dd > 0.0 && c2 > 1.0e-30) {
                const V3<double> cc = p - tn * dd;
                const double area = circle_triangle_area<double>(tn, a - cc, b - cc, c - cc, std::sqrt(c2));
                const double s2 = area > 0.0 ? std::fmin(1.0, area / (kPi * c2)) : 0.0;
                ref = s2 > 1.0e-12 ? s2 : 0.0;
            }
        }
        if (!meet) {
            ++rejected;
            if (d.dist > 0.0 && d.c2 > 1.0e-30 && disk_beyond_an_edge(d.n, d.ra, d.rb, d.rc, d.c2)) ++by_edge;
            if (ref != 0.0) {
                if (++bad <= 5) std::printf("rejected with scale %.3e (kind %d)\n", ref, kind);
            }
        } else {
            ++kept;
        }
        if (ref != 0.0 && !meet) ++missed;
        if (sc != ref) {
            if (++bad <= 10) std::printf("area scale %.17g differs from the edge sum's %.17g\n", sc, ref);
        }
    }
    std::printf("rejected %ld (beyond an edge %ld) kept %ld bad %ld missed %ld\n", rejected, by_edge, kept, bad,
                missed);
    if (bad == 0 && missed == 0 && rejected > 100000 && by_edge > 20000) std::printf("ALL OK\n");
    return bad == 0 && missed == 0 ? 0 : 1;
}
