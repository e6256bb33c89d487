// ref_geometry_harness.cpp -- C entry point around the reference's own CPU
// sphere/triangle overlap-area routine (TEST INFRASTRUCTURE ONLY).
//
// Compiled together with the reference's src/contact_geometry.cpp, where it
// lies in the reference tree, into oracle/_ref/libref_geometry.so by
// oracle/reference_build.py.  Tests use it to check the oracle's
// restatement of the GPU disk/triangle area against reference-built code.
#include "contact_geometry.h"

extern "C" double ref_sphere_triangle_area(const double* center, double radius, const double* a, const double* b,
                                           const double* c)
{
    const vector3d p(center[0], center[1], center[2]);
    const vector3d va(a[0], a[1], a[2]), vb(b[0], b[1], b[2]), vc(c[0], c[1], c[2]);
    return contact_geometry::sphereTriangleIntersectionArea(p, radius, va, vb, vc);
}
