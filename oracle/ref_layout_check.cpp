// ref_layout_check.cpp -- compile-time proof that oracle/ref_cuda_layout.h
// restates the reference's kernel argument structures byte for byte
// (TEST INFRASTRUCTURE ONLY).
//
// oracle/reference_build.py compiles this file with -fsyntax-only against
// the reference's src/cuda headers where they lie; every static_assert
// compares one field's type and offset, and each structure's size.
#include <cstddef>
#include <type_traits>

#include "cuda_contact_backend.cuh"
#include "ref_cuda_layout.h"

#define REF_CHECK_FIELD(Mine, Theirs, type, name)                                                        \
    static_assert(offsetof(Mine, name) == offsetof(Theirs, name), #Mine "." #name " offset");            \
    static_assert(std::is_same<decltype(Mine::name), decltype(Theirs::name)>::value, #Mine "." #name " type");

#define P_CHECK(type, name) REF_CHECK_FIELD(RefParticles, GpuParticleArrays, type, name)
#define C_CHECK(type, name) REF_CHECK_FIELD(RefComponents, GpuComponentArrays, type, name)
#define W_CHECK(type, name) REF_CHECK_FIELD(RefWalls, GpuWallArrays, type, name)
#define G_CHECK(type, name) REF_CHECK_FIELD(RefGrid, GpuGridArrays, type, name)
#define B_CHECK(type, name) REF_CHECK_FIELD(RefBodyStates, GpuBodyStateArrays, type, name)
#define T_CHECK(type, name) REF_CHECK_FIELD(RefTriangles, GpuTriangleArrays, type, name)
#define M_CHECK(type, name) REF_CHECK_FIELD(RefMech, GpuMechanicalParams, type, name)
#define H_CHECK(type, name) REF_CHECK_FIELD(RefHistory, GpuContactHistory, type, name)
#define F_CHECK(type, name) REF_CHECK_FIELD(RefForces, GpuForceArrays, type, name)
#define TG_CHECK(type, name) REF_CHECK_FIELD(RefTriangleGrid, GpuTriangleGrid, type, name)

REF_PARTICLE_FIELDS(P_CHECK)
REF_COMPONENT_FIELDS(C_CHECK)
REF_WALL_FIELDS(W_CHECK)
REF_GRID_FIELDS(G_CHECK)
REF_BODY_FIELDS(B_CHECK)
REF_TRIANGLE_FIELDS(T_CHECK)
REF_MECH_FIELDS(M_CHECK)
REF_HISTORY_FIELDS(H_CHECK)
REF_FORCE_FIELDS(F_CHECK)
REF_TRIANGLE_GRID_FIELDS(TG_CHECK)

static_assert(sizeof(RefParticles) == sizeof(GpuParticleArrays), "GpuParticleArrays size");
static_assert(sizeof(RefComponents) == sizeof(GpuComponentArrays), "GpuComponentArrays size");
static_assert(sizeof(RefWalls) == sizeof(GpuWallArrays), "GpuWallArrays size");
static_assert(sizeof(RefGrid) == sizeof(GpuGridArrays), "GpuGridArrays size");
static_assert(sizeof(RefBodyStates) == sizeof(GpuBodyStateArrays), "GpuBodyStateArrays size");
static_assert(sizeof(RefTriangles) == sizeof(GpuTriangleArrays), "GpuTriangleArrays size");
static_assert(sizeof(RefMech) == sizeof(GpuMechanicalParams), "GpuMechanicalParams size");
static_assert(sizeof(RefHistory) == sizeof(GpuContactHistory), "GpuContactHistory size");
static_assert(sizeof(RefForces) == sizeof(GpuForceArrays), "GpuForceArrays size");
static_assert(sizeof(RefTriangleGrid) == sizeof(GpuTriangleGrid), "GpuTriangleGrid size");

static_assert(REF_PARTICLE_SLOTS == kGpuParticleHistorySlots, "particle slots");
static_assert(REF_WALL_SLOTS == kGpuWallHistorySlots, "wall slots");
static_assert(REF_BODY_SLOTS == kGpuBodyHistorySlots, "body slots");
static_assert(REF_REGIME_COUNTERS == kGpuBodyRegimeCounterCount, "regime counters");
static_assert(REF_MICROSTATE_VALUES == kGpuBodyMicrostateValueCount, "microstate values");
