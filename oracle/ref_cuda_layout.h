/*
 * ref_cuda_layout.h -- the argument structures of the reference's CUDA
 * kernels, restated so that oracle/ref_cuda_host.cu can launch the
 * reference-built device code (TEST INFRASTRUCTURE ONLY).
 *
 * A kernel argument is passed byte for byte, so each structure must have the
 * reference's field types, order and offsets.  oracle/ref_layout_check.cpp
 * asserts that against the reference's own headers at build time:
 *   RefParticles      GpuParticleArrays   src/cuda/cuda_particle_backend.cuh:5-54
 *   RefComponents     GpuComponentArrays  src/cuda/cuda_particle_backend.cuh:56-78
 *   RefWalls          GpuWallArrays       src/cuda/cuda_particle_backend.cuh:80-88
 *   RefGrid           GpuGridArrays       src/cuda/cuda_grid_backend.cuh:8-14
 *   RefBodyStates     GpuBodyStateArrays  src/cuda/cuda_body_backend.cuh:5-20
 *   RefTriangles      GpuTriangleArrays   src/cuda/cuda_body_backend.cuh:22-65
 *   RefMech           GpuMechanicalParams src/cuda/cuda_contact_backend.cuh:24-39
 *   RefHistory        GpuContactHistory   src/cuda/cuda_contact_backend.cuh:41-52
 *   RefForces         GpuForceArrays      src/cuda/cuda_contact_backend.cuh:54-78
 *   RefTriangleGrid   GpuTriangleGrid     src/cuda/cuda_contact_backend.cuh:80-91
 * Field names follow the reference so the check can name each one.
 */
#ifndef REF_CUDA_LAYOUT_H
#define REF_CUDA_LAYOUT_H

#include <stdint.h>

#define REF_PARTICLE_FIELDS(X)                                                                           \
    X(int, n) X(double*, mass) X(double*, inertiaX) X(double*, inertiaY) X(double*, inertiaZ)            \
    X(double*, radius) X(int*, id) X(int*, status)                                                       \
    X(double*, x) X(double*, y) X(double*, z) X(double*, vx) X(double*, vy) X(double*, vz)               \
    X(double*, wx) X(double*, wy) X(double*, wz) X(double*, qw) X(double*, qx) X(double*, qy)            \
    X(double*, qz) X(double*, fx) X(double*, fy) X(double*, fz) X(double*, tx) X(double*, ty)            \
    X(double*, tz) X(double*, ax) X(double*, ay) X(double*, az) X(double*, awx) X(double*, awy)          \
    X(double*, awz) X(double*, vhx) X(double*, vhy) X(double*, vhz) X(double*, whx) X(double*, why)      \
    X(double*, whz) X(double*, hdqw) X(double*, hdqx) X(double*, hdqy) X(double*, hdqz)                  \
    X(double*, displacement)

#define REF_COMPONENT_FIELDS(X)                                                                          \
    X(int, n) X(int, ownerCount) X(int*, id) X(int*, owner) X(int*, ownerStart) X(double*, radius)       \
    X(double*, bodyX) X(double*, bodyY) X(double*, bodyZ) X(double*, offsetX) X(double*, offsetY)        \
    X(double*, offsetZ) X(double*, x) X(double*, y) X(double*, z) X(double*, vx) X(double*, vy)          \
    X(double*, vz) X(double*, vhx) X(double*, vhy) X(double*, vhz)

#define REF_WALL_FIELDS(X)                                                                               \
    X(int, n) X(double*, ox) X(double*, oy) X(double*, oz) X(double*, nx) X(double*, ny) X(double*, nz)

#define REF_GRID_FIELDS(X)                                                                               \
    X(int, n) X(double, invMeshSize) X(uint64_t*, sortedCellKey) X(int*, sortedEntityId)                 \
    X(int*, overflowCount)

#define REF_BODY_FIELDS(X)                                                                               \
    X(int, n) X(double*, cx) X(double*, cy) X(double*, cz) X(double*, qw) X(double*, qx) X(double*, qy)  \
    X(double*, qz) X(double*, vx) X(double*, vy) X(double*, vz) X(double*, wx) X(double*, wy)            \
    X(double*, wz)

#define REF_TRIANGLE_FIELDS(X)                                                                           \
    X(int, n) X(int*, bodyId) X(int*, triId)                                                             \
    X(double*, lx1) X(double*, ly1) X(double*, lz1) X(double*, lx2) X(double*, ly2) X(double*, lz2)      \
    X(double*, lx3) X(double*, ly3) X(double*, lz3) X(double*, lx4) X(double*, ly4) X(double*, lz4)      \
    X(double*, lnx) X(double*, lny) X(double*, lnz)                                                      \
    X(double*, wx1) X(double*, wy1) X(double*, wz1) X(double*, wx2) X(double*, wy2) X(double*, wz2)      \
    X(double*, wx3) X(double*, wy3) X(double*, wz3) X(double*, wx4) X(double*, wy4) X(double*, wz4)      \
    X(double*, wnx) X(double*, wny) X(double*, wnz)                                                      \
    X(double*, aabbMinX) X(double*, aabbMinY) X(double*, aabbMinZ)                                       \
    X(double*, aabbMaxX) X(double*, aabbMaxY) X(double*, aabbMaxZ)

#define REF_MECH_FIELDS(X)                                                                               \
    X(double, epsS) X(double, mu) X(double, epsN) X(double, cohesion) X(double, beta) X(double, muT)     \
    X(double, muR) X(double, kN) X(double, dt) X(double, gx) X(double, gy) X(double, gz)                 \
    X(int, gravityEnabled) X(int, universalGravityEnabled)

#define REF_HISTORY_FIELDS(X)                                                                            \
    X(int, particleCount) X(uint64_t*, particleKeys) X(uint64_t*, wallKeys) X(uint64_t*, bodyKeys)       \
    X(int*, particleLastSeen) X(int*, wallLastSeen) X(int*, bodyLastSeen) X(double*, particleValues)     \
    X(double*, wallValues) X(double*, bodyValues)

#define REF_FORCE_FIELDS(X)                                                                              \
    X(int, particleCount) X(int, componentCount) X(int, bodyCount) X(double*, contact)                   \
    X(double*, field) X(double*, wall) X(double*, total) X(double*, bodyParticle)                        \
    X(double*, bodyDetail) X(double*, bodyResult) X(int*, particleContactCount)                          \
    X(int*, bodyContactCount) X(int*, particleHistoryOverflowCount) X(int*, bodyHistoryOverflowCount)    \
    X(int*, particleHistoryHighWater) X(int*, bodyHistoryHighWater) X(double*, bodyMaxDepth)             \
    X(double*, bodyContactFz) X(int*, bodyRegimeState) X(unsigned long long*, bodyRegimeInstant)         \
    X(unsigned long long*, bodyRegimeInterval) X(double*, bodyMicrostateState)                          \
    X(double*, bodyMicrostateInstant) X(double*, bodyMicrostateInterval)

#define REF_TRIANGLE_GRID_FIELDS(X)                                                                      \
    X(int, triangleCount) X(int, capacity) X(int, entryCount) X(double, invMeshSize) X(double, padding)  \
    X(int*, counts) X(int*, offsets) X(uint64_t*, sortedCellKey) X(int*, sortedTriangleId)               \
    X(int*, overflowCount)

#define REF_DECLARE_FIELD(type, name) type name;

struct RefParticles { REF_PARTICLE_FIELDS(REF_DECLARE_FIELD) };
struct RefComponents { REF_COMPONENT_FIELDS(REF_DECLARE_FIELD) };
struct RefWalls { REF_WALL_FIELDS(REF_DECLARE_FIELD) };
struct RefGrid { REF_GRID_FIELDS(REF_DECLARE_FIELD) };
struct RefBodyStates { REF_BODY_FIELDS(REF_DECLARE_FIELD) };
struct RefTriangles { REF_TRIANGLE_FIELDS(REF_DECLARE_FIELD) };
struct RefMech { REF_MECH_FIELDS(REF_DECLARE_FIELD) };
struct RefHistory { REF_HISTORY_FIELDS(REF_DECLARE_FIELD) };
struct RefForces { REF_FORCE_FIELDS(REF_DECLARE_FIELD) };
struct RefTriangleGrid { REF_TRIANGLE_GRID_FIELDS(REF_DECLARE_FIELD) };

/* Slot counts and diagnostic sizes (src/cuda/cuda_contact_backend.cuh:11-16). */
enum {
    REF_PARTICLE_SLOTS = 64,
    REF_WALL_SLOTS = 16,
    REF_BODY_SLOTS = 64,
    REF_REGIME_COUNTERS = 7,
    REF_MICROSTATE_VALUES = 22
};

#endif
