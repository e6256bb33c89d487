/*
 * dem_oracle.c -- CPU FP64 restatement of the reference DEM step (TEST
 * INFRASTRUCTURE ONLY).
 *
 * This file is the correctness oracle of the GB300 engine.  It restates, in
 * plain C99 and double precision, the algorithm of the reference's GPU DEM
 * step engine so that tests can compare the CUDA engine with it on the same
 * seeded inputs.  It is never linked into the engine and the engine never
 * calls it; only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py load it.
 *
 * Every function names the reference file:line it follows.  The data layout
 * deliberately mirrors the reference (input-order SoA, per-component history
 * slot arrays, a sorted (cell key, entity id) list searched by binary search)
 * because the oracle's job is to reproduce the reference's results, not to be
 * fast.  Parity pins: the reference's own known-answer tests
 * (tests/scenario_validator.cpp:80-113, tests/contact_geometry_test.cpp:37-72,
 * tests/component_transform_test.cu:45-113) are re-run against this file by
 * tests/test_oracle_golden.py.
 *
 * Build: cc -O2 -std=gnu99 -ffp-contract=off -fopenmp -shared -fPIC.
 * Contraction is disabled so results are identical on x86-64 and AArch64;
 * the overlap predicate alone uses an explicit fma() in the evaluation order
 * the CUDA compiler uses for a*b + c*d + e*f (see pp_distance_squared).
 */
#include "../include/dem_gb300.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.1415926535897932384626433832795
#define ORC_G 6.67430e-11
#define PSLOTS DEM_PARTICLE_HISTORY_SLOTS
#define WSLOTS DEM_WALL_HISTORY_SLOTS
#define BSLOTS DEM_BODY_HISTORY_SLOTS
#define NREG DEM_BODY_REGIME_COUNTERS
#define NMICRO DEM_BODY_MICROSTATE_VALUES

static char g_error[512];
static void set_error(const char* msg) { snprintf(g_error, sizeof g_error, "%s", msg); }
const char* orc_error(void) { return g_error; }

/* ------------------------------------------------------------------ vectors */
typedef struct { double x, y, z; } v3;
typedef struct { double x, y; } v2;
static v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 mul(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 cross(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static double norm(v3 a) { return sqrt(dot(a, a)); }
/* src/cuda/cuda_contact_backend.cu:68-72 */
static v3 normalized(v3 a) { double l = norm(a); return l > 1.0e-14 ? mul(a, 1.0 / l) : mk(0, 0, 0); }
static v3 ld3(const double* p, long i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
static void st3(double* p, long i, v3 v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }

/* Overlap predicate operand: the reference computes normSquared(delta) =
 * dx*dx + dy*dy + dz*dz (src/cuda/cuda_contact_backend.cu:593) and nvcc
 * contracts it to fma(dz,dz, fma(dy,dy, dx*dx)).  The oracle spells that out
 * so the contact set is decided by the same bits on every host. */
static double pp_distance_squared(v3 d) { return fma(d.z, d.z, fma(d.y, d.y, d.x * d.x)); }

/* rotateIv / rotateBodyToWorld / rotateByQuatIv: Quat2IvDCM convention
 * (src/cuda/cuda_contact_backend.cu:109-116, cuda_particle_backend.cu:103-114). */
static v3 rot_iv(const double* q, v3 v)
{
    double qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    return mk((1.0 - 2.0 * (qy * qy + qz * qz)) * v.x + 2.0 * (qx * qy - qw * qz) * v.y + 2.0 * (qx * qz + qw * qy) * v.z,
              2.0 * (qx * qy + qw * qz) * v.x + (1.0 - 2.0 * (qx * qx + qz * qz)) * v.y + 2.0 * (qy * qz - qw * qx) * v.z,
              2.0 * (qx * qz - qw * qy) * v.x + 2.0 * (qy * qz + qw * qx) * v.y + (1.0 - 2.0 * (qx * qx + qy * qy)) * v.z);
}
/* src/cuda/cuda_body_backend.cu:25-50 (same matrix, precomputed entries) */
static v3 rot_iv_body(const double* q, v3 v)
{
    double qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    double r00 = 1.0 - 2.0 * (qy * qy + qz * qz), r01 = 2.0 * (qx * qy - qw * qz), r02 = 2.0 * (qx * qz + qw * qy);
    double r10 = 2.0 * (qx * qy + qw * qz), r11 = 1.0 - 2.0 * (qx * qx + qz * qz), r12 = 2.0 * (qy * qz - qw * qx);
    double r20 = 2.0 * (qx * qz - qw * qy), r21 = 2.0 * (qy * qz + qw * qx), r22 = 1.0 - 2.0 * (qx * qx + qy * qy);
    return mk(r00 * v.x + r01 * v.y + r02 * v.z, r10 * v.x + r11 * v.y + r12 * v.z, r20 * v.x + r21 * v.y + r22 * v.z);
}

/* packCell (src/cuda/cuda_grid_backend.cu:19-26) */
static uint64_t pack_cell(int x, int y, int z)
{
    const int bias = 1 << 20;
    const uint64_t m = (1ull << 21) - 1ull;
    return (((uint64_t)(int64_t)(x + bias) & m) << 42) | (((uint64_t)(int64_t)(y + bias) & m) << 21) |
           ((uint64_t)(int64_t)(z + bias) & m);
}

/* lowerBound / upperBound (src/cuda/cuda_contact_backend.cu:144-176) */
static int lower_bound_u64(const uint64_t* k, int n, uint64_t key)
{
    int first = 0, len = n;
    while (len > 0) { int h = len >> 1, m = first + h; if (k[m] < key) { first = m + 1; len -= h + 1; } else len = h; }
    return first;
}
static int upper_bound_u64(const uint64_t* k, int n, uint64_t key)
{
    int first = 0, len = n;
    while (len > 0) { int h = len >> 1, m = first + h; if (key < k[m]) len = h; else { first = m + 1; len -= h + 1; } }
    return first;
}

/* -------------------------------------------------------------------- state */
typedef struct {
    double epsS, mu, epsN, cohesion, beta, muT, muR, kN, dt;
} mech_t;

typedef struct {
    uint64_t* keys;
    int* last;
    double* val; /* [slot][roll, tangent, twist][xyz] */
    int slots;
} hist_t;

typedef struct orc {
    int n, nc, nw, nb, nt, nthreads;
    /* owners, input order (src/cuda/cuda_particle_backend.cuh:5-54) */
    int *id, *status;
    double *mass, *inertia, *radius;
    double *pos, *vel, *omg, *quat, *f, *t, *acc, *aacc, *vh, *wh, *hdq;
    /* components (src/cuda/cuda_particle_backend.cuh:56-78) */
    int *cid, *cowner, *ostart;
    double *crad, *cbody, *coff, *cpos, *cvel, *cvh;
    /* walls */
    double *wo, *wn;
    /* bodies: per-step device copy of the host state */
    double *bc, *bq, *bv, *bw;
    double *bmass, *binertia;
    int* bstate;
    /* triangles (src/cuda/cuda_body_backend.cuh:22-70) */
    int* tbody;
    double *tloc, *tw; /* tw: [t][15] world v1..v4, normal */
    double* taabb;     /* [t][6] */
    /* particle grid */
    uint64_t* skey;
    int* sid;
    double inv_mesh, mesh, max_radius;
    /* triangle grid */
    int tcap, tentries;
    uint64_t* tkey;
    int* tid;
    /* history */
    hist_t hp, hw, hb;
    /* forces (GpuForceArrays, src/cuda/cuda_contact_backend.cuh:54-80) */
    double *fcontact, *ffield, *fwall, *ftotal, *fbodyp, *fbodyd;
    double* bres;
    int pcontacts, bcontacts, pover, bover, phigh, bhigh, tgover;
    double bmaxdepth, bfz;
    int* regime_state;
    unsigned long long *reg_inst, *reg_int;
    double *micro_state, *micro_inst, *micro_int;
    unsigned long long reg_native_steps;
    /* the copies the last diagnostic evaluation downloaded */
    unsigned long long *diag_reg_inst, *diag_reg_int;
    double *diag_micro_inst, *diag_micro_int;
    mech_t pp, pt, pw;
    double g[3];
    int grav, ugrav;
    int step_index;
    /* cached stats of the last diagnostic evaluation */
    dem_step_stats stats;
    /* host MBD driver (src/cuda_simulation_integrator.cpp:288-446) */
    int started, restored_leapfrog;
    int drv_step;
    double *bhalf_v, *bhalf_w, *bhalf_q, *bhalf_dq, *bacc, *bdomg, *bloads;
} orc;

static void* zalloc(size_t n) { void* p = calloc(n ? n : 1, 1); return p; }

static void hist_alloc(hist_t* h, int nc, int slots)
{
    size_t s = (size_t)nc * slots;
    h->slots = slots;
    h->keys = zalloc(s * sizeof(uint64_t));
    h->last = malloc(s * sizeof(int));
    for (size_t i = 0; i < s; ++i) h->last[i] = -1;
    h->val = zalloc(s * 9 * sizeof(double));
}
static void hist_free(hist_t* h) { free(h->keys); free(h->last); free(h->val); }

static mech_t to_mech(dem_mech m, double dt)
{
    mech_t r = {m.epsS, m.mu, m.epsN, m.cohesion, m.beta, m.muT, m.muR, m.kN, dt};
    return r;
}

void orc_destroy(orc* o);

/* CudaDemSolver::initialize (src/cuda_backend_cuda.cu:302-381) including
 * uploadComponents (:121-190). */
orc* orc_create(const dem_scene* s, int nthreads)
{
    if (!s || s->n_owners <= 0) { set_error("scene requires particles"); return NULL; }
    orc* o = zalloc(sizeof(orc));
    int n = s->n_owners;
    o->n = n;
    o->nthreads = nthreads > 0 ? nthreads : 1;
    o->id = malloc(n * sizeof(int)); memcpy(o->id, s->owner_id, n * sizeof(int));
    o->status = malloc(n * sizeof(int)); memcpy(o->status, s->owner_status, n * sizeof(int));
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i && n < 5000; ++j)
            if (o->id[i] == o->id[j]) { set_error("duplicate particle ID"); orc_destroy(o); return NULL; }
#define CP(dst, src, cnt) do { dst = malloc((size_t)(cnt) * sizeof(double)); memcpy(dst, src, (size_t)(cnt) * sizeof(double)); } while (0)
    CP(o->mass, s->owner_mass, n);
    CP(o->radius, s->owner_radius, n);
    CP(o->inertia, s->owner_inertia, 3 * n);
    CP(o->pos, s->owner_pos, 3 * n);
    CP(o->vel, s->owner_vel, 3 * n);
    CP(o->omg, s->owner_omega, 3 * n);
    CP(o->quat, s->owner_quat, 4 * n);
    o->f = zalloc(3 * n * sizeof(double)); o->t = zalloc(3 * n * sizeof(double));
    o->acc = zalloc(3 * n * sizeof(double)); o->aacc = zalloc(3 * n * sizeof(double));
    o->vh = zalloc(3 * n * sizeof(double)); o->wh = zalloc(3 * n * sizeof(double));
    o->hdq = zalloc(4 * n * sizeof(double));

    /* components sorted by (owner, component id) */
    int nc = s->n_components > 0 ? s->n_components : n;
    o->nc = nc;
    int* order = malloc(nc * sizeof(int));
    int* in_owner = malloc(nc * sizeof(int));
    int* in_id = malloc(nc * sizeof(int));
    double* in_rad = malloc(nc * sizeof(double));
    double* in_off = zalloc(3 * nc * sizeof(double));
    for (int c = 0; c < nc; ++c) {
        if (s->n_components > 0) {
            in_owner[c] = s->comp_owner[c]; in_id[c] = s->comp_id[c]; in_rad[c] = s->comp_radius[c];
            in_off[3 * c] = s->comp_offset[3 * c]; in_off[3 * c + 1] = s->comp_offset[3 * c + 1]; in_off[3 * c + 2] = s->comp_offset[3 * c + 2];
        } else {
            in_owner[c] = c; in_id[c] = s->owner_id[c]; in_rad[c] = s->owner_radius[c];
        }
        order[c] = c;
    }
    /* insertion-free sort by (owner, id): simple O(nc log nc) merge via qsort on packed pairs */
    {
        int64_t* packed = malloc(nc * sizeof(int64_t));
        for (int c = 0; c < nc; ++c) packed[c] = ((int64_t)in_owner[c] << 32) | (int64_t)(uint32_t)c;
        /* stable order by owner then id: sort indices with comparator */
        for (int c = 0; c < nc; ++c) order[c] = c;
        /* shell sort on comparator (owner, id) -- nc is small for clumps, spheres are already ordered */
        int sorted = 1;
        for (int c = 1; c < nc && sorted; ++c)
            if (in_owner[order[c - 1]] > in_owner[order[c]] ||
                (in_owner[order[c - 1]] == in_owner[order[c]] && in_id[order[c - 1]] > in_id[order[c]])) sorted = 0;
        if (!sorted) {
            for (int gap = nc / 2; gap > 0; gap /= 2)
                for (int c = gap; c < nc; ++c) {
                    int tmp = order[c], j = c;
                    while (j >= gap && (in_owner[order[j - gap]] > in_owner[tmp] ||
                                        (in_owner[order[j - gap]] == in_owner[tmp] && in_id[order[j - gap]] > in_id[tmp]))) {
                        order[j] = order[j - gap]; j -= gap;
                    }
                    order[j] = tmp;
                }
        }
        free(packed);
    }
    o->cid = malloc(nc * sizeof(int)); o->cowner = malloc(nc * sizeof(int));
    o->ostart = zalloc((n + 1) * sizeof(int));
    o->crad = malloc(nc * sizeof(double)); o->cbody = zalloc(3 * nc * sizeof(double));
    o->coff = zalloc(3 * nc * sizeof(double)); o->cpos = zalloc(3 * nc * sizeof(double));
    o->cvel = zalloc(3 * nc * sizeof(double)); o->cvh = zalloc(3 * nc * sizeof(double));
    double max_r = 0.0;
    for (int k = 0; k < nc; ++k) {
        int c = order[k];
        if (in_owner[c] < 0 || in_owner[c] >= n || in_id[c] < 0 || !(in_rad[c] > 0.0) || !isfinite(in_rad[c])) {
            set_error("invalid native clump component topology");
            free(order); free(in_owner); free(in_id); free(in_rad); free(in_off); orc_destroy(o); return NULL;
        }
        o->cid[k] = in_id[c]; o->cowner[k] = in_owner[c]; o->crad[k] = in_rad[c];
        o->cbody[3 * k] = in_off[3 * c]; o->cbody[3 * k + 1] = in_off[3 * c + 1]; o->cbody[3 * k + 2] = in_off[3 * c + 2];
        o->ostart[in_owner[c] + 1]++;
        if (in_rad[c] > max_r) max_r = in_rad[c];
    }
    for (int i = 1; i <= n; ++i) {
        o->ostart[i] += o->ostart[i - 1];
        int cnt = o->ostart[i] - o->ostart[i - 1];
        if (cnt < 1 || cnt > 8) {
            set_error("each owner requires 1 to 8 components");
            free(order); free(in_owner); free(in_id); free(in_rad); free(in_off); orc_destroy(o); return NULL;
        }
    }
    free(order); free(in_owner); free(in_id); free(in_rad); free(in_off);
    o->skey = zalloc(nc * sizeof(uint64_t));
    o->sid = zalloc(nc * sizeof(int));
    hist_alloc(&o->hp, nc, PSLOTS);
    hist_alloc(&o->hw, nc, WSLOTS);
    hist_alloc(&o->hb, nc, BSLOTS);

    o->nw = s->n_walls;
    if (o->nw > 0) { CP(o->wo, s->wall_origin, 3 * o->nw); CP(o->wn, s->wall_normal, 3 * o->nw); }
    o->nb = s->n_bodies;
    o->nt = s->n_bodies > 0 ? s->n_triangles : 0;
    int nb = o->nb;
    if (nb > 0) {
        CP(o->bc, s->body_center, 3 * nb); CP(o->bq, s->body_quat, 4 * nb);
        CP(o->bv, s->body_vel, 3 * nb); CP(o->bw, s->body_omega, 3 * nb);
        CP(o->bmass, s->body_mass, nb); CP(o->binertia, s->body_inertia, 9 * nb);
        o->bstate = malloc(nb * sizeof(int)); memcpy(o->bstate, s->body_state, nb * sizeof(int));
        if (o->nt > 0) {
            o->tbody = malloc(o->nt * sizeof(int)); memcpy(o->tbody, s->tri_body, o->nt * sizeof(int));
            CP(o->tloc, s->tri_local, 15 * o->nt);
            o->tw = zalloc(15 * o->nt * sizeof(double));
            o->taabb = zalloc(6 * o->nt * sizeof(double));
        }
        o->regime_state = zalloc((size_t)nb * nc * sizeof(int));
        o->reg_inst = zalloc((size_t)nb * NREG * sizeof(unsigned long long));
        o->reg_int = zalloc((size_t)nb * NREG * sizeof(unsigned long long));
        o->micro_state = zalloc((size_t)nb * nc * NMICRO * sizeof(double));
        o->micro_inst = zalloc((size_t)nb * NMICRO * sizeof(double));
        o->micro_int = zalloc((size_t)nb * NMICRO * sizeof(double));
        o->diag_reg_inst = zalloc((size_t)nb * NREG * sizeof(unsigned long long));
        o->diag_reg_int = zalloc((size_t)nb * NREG * sizeof(unsigned long long));
        o->diag_micro_inst = zalloc((size_t)nb * NMICRO * sizeof(double));
        o->diag_micro_int = zalloc((size_t)nb * NMICRO * sizeof(double));
        o->bhalf_v = zalloc(3 * nb * sizeof(double)); o->bhalf_w = zalloc(3 * nb * sizeof(double));
        o->bhalf_q = zalloc(4 * nb * sizeof(double)); o->bhalf_dq = zalloc(4 * nb * sizeof(double));
        o->bacc = zalloc(3 * nb * sizeof(double)); o->bdomg = zalloc(3 * nb * sizeof(double));
        o->bloads = zalloc(6 * nb * sizeof(double));
    }
#undef CP
    o->fcontact = zalloc(6 * (size_t)n * sizeof(double)); o->ffield = zalloc(6 * (size_t)n * sizeof(double));
    o->fwall = zalloc(6 * (size_t)n * sizeof(double)); o->ftotal = zalloc(6 * (size_t)n * sizeof(double));
    if (s->keep_body_particle && nb > 0) o->fbodyp = zalloc((size_t)nb * n * 6 * sizeof(double));
    if (s->keep_body_detail && nb > 0) o->fbodyd = zalloc((size_t)nb * n * 19 * sizeof(double));
    o->bres = zalloc((nb > 0 ? nb : 1) * 6 * sizeof(double));
    o->pp = to_mech(s->pp, s->dt); o->pt = to_mech(s->pt, s->dt); o->pw = to_mech(s->pw, s->dt);
    o->g[0] = s->gravity[0]; o->g[1] = s->gravity[1]; o->g[2] = s->gravity[2];
    o->grav = s->gravity_enabled; o->ugrav = s->universal_gravity_enabled;
    o->max_radius = max_r;
    o->mesh = 2.5 * max_r;
    o->inv_mesh = 1.0 / o->mesh;
    return o;
}

void orc_destroy(orc* o)
{
    if (!o) return;
    void* ptrs[] = {o->id, o->status, o->mass, o->inertia, o->radius, o->pos, o->vel, o->omg, o->quat, o->f, o->t,
                    o->acc, o->aacc, o->vh, o->wh, o->hdq, o->cid, o->cowner, o->ostart, o->crad, o->cbody, o->coff,
                    o->cpos, o->cvel, o->cvh, o->wo, o->wn, o->bc, o->bq, o->bv, o->bw, o->bmass, o->binertia,
                    o->bstate, o->tbody, o->tloc, o->tw, o->taabb, o->skey, o->sid, o->tkey, o->tid, o->fcontact,
                    o->ffield, o->fwall, o->ftotal, o->fbodyp, o->fbodyd, o->bres, o->regime_state, o->reg_inst,
                    o->reg_int, o->micro_state, o->micro_inst, o->micro_int, o->bhalf_v, o->bhalf_w, o->bhalf_q,
                    o->bhalf_dq, o->bacc, o->bdomg, o->bloads, o->diag_reg_inst, o->diag_reg_int,
                    o->diag_micro_inst, o->diag_micro_int};
    for (size_t k = 0; k < sizeof ptrs / sizeof ptrs[0]; ++k) free(ptrs[k]);
    hist_free(&o->hp); hist_free(&o->hw); hist_free(&o->hb);
    free(o);
}

/* ------------------------------------------------------------- components */
/* updateComponentsKernel (src/cuda/cuda_particle_backend.cu:116-147) */
static void update_components(orc* o)
{
    for (int c = 0; c < o->nc; ++c) {
        int w = o->cowner[c];
        const double* q = o->quat + 4 * w;
        v3 off = rot_iv(q, ld3(o->cbody, c));
        st3(o->coff, c, off);
        st3(o->cpos, c, add(ld3(o->pos, w), off));
        v3 ow = rot_iv(q, ld3(o->omg, w));
        v3 v = ld3(o->vel, w);
        st3(o->cvel, c, mk(v.x + (ow.y * off.z - ow.z * off.y), v.y + (ow.z * off.x - ow.x * off.z), v.z + (ow.x * off.y - ow.y * off.x)));
        v3 hw = rot_iv(q, ld3(o->wh, w));
        v3 hv = ld3(o->vh, w);
        st3(o->cvh, c, mk(hv.x + (hw.y * off.z - hw.z * off.y), hv.y + (hw.z * off.x - hw.x * off.z), hv.z + (hw.x * off.y - hw.y * off.x)));
    }
}

/* ------------------------------------------------------------------- grids */
static const uint64_t* g_sort_keys;
static int cmp_key_then_index(const void* a, const void* b)
{
    int ia = *(const int*)a, ib = *(const int*)b;
    uint64_t ka = g_sort_keys[ia], kb = g_sort_keys[ib];
    if (ka < kb) return -1;
    if (ka > kb) return 1;
    return (ia > ib) - (ia < ib);
}

/* gpuBuildComponentGrid + computeComponentKeysKernel
 * (src/cuda/cuda_grid_backend.cu:51-71,121-145): stable sort of cell keys
 * over component indices 0..nc-1. */
static int build_particle_grid(orc* o)
{
    const double minCell = -(double)(1 << 20), maxCell = (double)((1 << 20) - 1);
    uint64_t* keys = malloc(o->nc * sizeof(uint64_t));
    int overflow = 0;
    for (int c = 0; c < o->nc; ++c) {
        double cx = floor(o->cpos[3 * c] * o->inv_mesh);
        double cy = floor(o->cpos[3 * c + 1] * o->inv_mesh);
        double cz = floor(o->cpos[3 * c + 2] * o->inv_mesh);
        if (!isfinite(cx) || !isfinite(cy) || !isfinite(cz) || cx < minCell || cx > maxCell || cy < minCell ||
            cy > maxCell || cz < minCell || cz > maxCell) {
            overflow++; keys[c] = 0; continue;
        }
        keys[c] = pack_cell((int)cx, (int)cy, (int)cz);
    }
    if (overflow) { free(keys); set_error("component grid coordinate exceeds signed 21-bit hash range"); return DEM_ERR_CAPACITY; }
    for (int c = 0; c < o->nc; ++c) o->sid[c] = c;
    g_sort_keys = keys;
    qsort(o->sid, o->nc, sizeof(int), cmp_key_then_index);
    for (int k = 0; k < o->nc; ++k) o->skey[k] = keys[o->sid[k]];
    free(keys);
    return DEM_OK;
}

/* transformTrianglesKernel (src/cuda/cuda_body_backend.cu:71-112) */
static void transform_triangles(orc* o)
{
    for (int i = 0; i < o->nt; ++i) {
        int b = o->tbody[i];
        const double* q = o->bq + 4 * b;
        const double* L = o->tloc + 15 * i;
        double* W = o->tw + 15 * i;
        v3 c = ld3(o->bc, b);
        for (int k = 0; k < 4; ++k) {
            v3 p = rot_iv_body(q, mk(L[3 * k], L[3 * k + 1], L[3 * k + 2]));
            p = mk(p.x + c.x, p.y + c.y, p.z + c.z);
            W[3 * k] = p.x; W[3 * k + 1] = p.y; W[3 * k + 2] = p.z;
        }
        v3 nn = rot_iv_body(q, mk(L[12], L[13], L[14]));
        W[12] = nn.x; W[13] = nn.y; W[14] = nn.z;
        double* A = o->taabb + 6 * i;
        A[0] = W[0]; A[1] = W[1]; A[2] = W[2]; A[3] = W[0]; A[4] = W[1]; A[5] = W[2];
        for (int k = 1; k < 4; ++k) {
            A[0] = fmin(A[0], W[3 * k]); A[1] = fmin(A[1], W[3 * k + 1]); A[2] = fmin(A[2], W[3 * k + 2]);
            A[3] = fmax(A[3], W[3 * k]); A[4] = fmax(A[4], W[3 * k + 1]); A[5] = fmax(A[5], W[3 * k + 2]);
        }
    }
}

/* countTriangleCellsKernel + fillTriangleCellsKernel + gpuBuildTriangleGrid
 * (src/cuda/cuda_contact_backend.cu:409-476,1567-1610).  Entries of one
 * cell end up in ascending triangle order (stable sort of the fill order). */
static int build_triangle_grid(orc* o)
{
    o->tentries = 0;
    if (o->nt <= 0) return DEM_OK;
    const double pad = o->max_radius, inv = o->inv_mesh;
    const double minCell = -(double)(1 << 20), maxCell = (double)((1 << 20) - 1);
    long long* counts = zalloc(o->nt * sizeof(long long));
    int* lo = malloc(3 * o->nt * sizeof(int));
    int* hi = malloc(3 * o->nt * sizeof(int));
    unsigned long long total = 0;
    int overflow = 0;
    for (int i = 0; i < o->nt; ++i) {
        const double* A = o->taabb + 6 * i;
        double mn[3], mx[3];
        for (int a = 0; a < 3; ++a) { mn[a] = floor((A[a] - pad) * inv); mx[a] = floor((A[3 + a] + pad) * inv); }
        int bad = 0;
        for (int a = 0; a < 3; ++a)
            if (!isfinite(mn[a]) || !isfinite(mx[a]) || mn[a] < minCell || mx[a] > maxCell) bad = 1;
        if (bad) { overflow++; counts[i] = 0; continue; }
        long long nx = (long long)(int)mx[0] - (int)mn[0] + 1, ny = (long long)(int)mx[1] - (int)mn[1] + 1,
                  nz = (long long)(int)mx[2] - (int)mn[2] + 1;
        if (nx <= 0 || ny <= 0 || nz <= 0) { overflow++; counts[i] = 0; continue; }
        counts[i] = nx * ny * nz;
        for (int a = 0; a < 3; ++a) { lo[3 * i + a] = (int)mn[a]; hi[3 * i + a] = (int)mx[a]; }
        total += (unsigned long long)counts[i];
    }
    o->tgover = overflow;
    if (overflow || total > 2147483647ull) {
        free(counts); free(lo); free(hi);
        set_error("triangle grid entry count exceeds the supported 32-bit index range");
        return DEM_ERR_CAPACITY;
    }
    if ((int)total > o->tcap) {
        free(o->tkey); free(o->tid);
        o->tkey = malloc(total * sizeof(uint64_t)); o->tid = malloc(total * sizeof(int));
        o->tcap = (int)total;
    }
    uint64_t* keys = malloc((total ? total : 1) * sizeof(uint64_t));
    int* ids = malloc((total ? total : 1) * sizeof(int));
    long long e = 0;
    for (int i = 0; i < o->nt; ++i) {
        if (!counts[i]) continue;
        for (int x = lo[3 * i]; x <= hi[3 * i]; ++x)
            for (int y = lo[3 * i + 1]; y <= hi[3 * i + 1]; ++y)
                for (int z = lo[3 * i + 2]; z <= hi[3 * i + 2]; ++z) { keys[e] = pack_cell(x, y, z); ids[e] = i; ++e; }
    }
    int* perm = malloc((total ? total : 1) * sizeof(int));
    for (long long k = 0; k < (long long)total; ++k) perm[k] = (int)k;
    g_sort_keys = keys;
    qsort(perm, total, sizeof(int), cmp_key_then_index);
    for (long long k = 0; k < (long long)total; ++k) { o->tkey[k] = keys[perm[k]]; o->tid[k] = ids[perm[k]]; }
    o->tentries = (int)total;
    free(perm); free(keys); free(ids); free(counts); free(lo); free(hi);
    return DEM_OK;
}

/* ----------------------------------------------------------------- history */
typedef struct {
    int pover, bover, phigh, bhigh, pcontacts, bcontacts;
    double bmaxdepth, bfz;
    double* bres; /* [nb][6] partial */
} tls_t;

/* acquireHistorySlot (src/cuda/cuda_contact_backend.cu:190-215) */
static int acquire_slot(hist_t* h, int comp, uint64_t key, int step, int* overflow, int* high)
{
    const int begin = comp * h->slots;
    int empty = -1;
    for (int s = 0; s < h->slots; ++s) {
        int idx = begin + s;
        if (h->keys[idx] == key) {
            h->last[idx] = step;
            if (s + 1 > *high) *high = s + 1;
            return idx;
        }
        if (h->keys[idx] == 0 && empty < 0) empty = idx;
    }
    if (empty < 0) { (*overflow)++; return -1; }
    h->keys[empty] = key;
    h->last[empty] = step;
    for (int k = 0; k < 9; ++k) h->val[(size_t)empty * 9 + k] = 0.0;
    if (empty - begin + 1 > *high) *high = empty - begin + 1;
    return empty;
}

/* expireHistory (src/cuda/cuda_contact_backend.cu:217-229) */
static void expire(hist_t* h, int comp, int step)
{
    const int begin = comp * h->slots;
    for (int s = 0; s < h->slots; ++s) {
        int idx = begin + s;
        if (h->keys[idx] != 0 && h->last[idx] < step - 1) {
            h->keys[idx] = 0; h->last[idx] = -1;
            for (int k = 0; k < 9; ++k) h->val[(size_t)idx * 9 + k] = 0.0;
        }
    }
}

static v3 hload(const hist_t* h, int slot, int cat) { const double* p = h->val + (size_t)slot * 9 + cat * 3; return mk(p[0], p[1], p[2]); }
static void hstore(hist_t* h, int slot, int cat, v3 v) { double* p = h->val + (size_t)slot * 9 + cat * 3; p[0] = v.x; p[1] = v.y; p[2] = v.z; }

/* transportTangentHistory / transportAxialHistory (:245-265) */
static v3 transport_tangent(v3 prev, v3 n)
{
    double pn = norm(prev);
    v3 proj = sub(prev, mul(n, dot(prev, n)));
    double qn = norm(proj);
    if (pn <= 1.0e-30 || qn <= 1.0e-30) return mk(0, 0, 0);
    return mul(proj, pn / qn);
}
static v3 transport_axial(v3 prev, v3 n)
{
    double pn = norm(prev);
    if (pn <= 1.0e-30) return mk(0, 0, 0);
    double al = dot(prev, n);
    if (fabs(al) <= 1.0e-30) return mk(0, 0, 0);
    return mul(n, al < 0.0 ? -pn : pn);
}

/* limitedHistoryResponseRates (:267-299) */
static v3 limited_rates(v3 hrate, v3 rrate, double k, double c, double dt, v3 prev, double limit, hist_t* h, int slot,
                        int cat, int store, int* yielded)
{
    v3 delta = mul(hrate, dt);
    v3 inc = mul(delta, k);
    v3 et = add(inc, prev);
    v3 trial = add(mul(rrate, c), et);
    double tn = norm(et);
    v3 resp;
    int y = tn > limit;
    if (yielded) *yielded = y;
    if (y) {
        double dn = norm(delta);
        if (dn > 1.0e-14) resp = mul(et, limit / tn);
        else {
            double pn = norm(prev);
            resp = pn > 1.0e-14 ? mul(prev, limit / pn) : mk(0, 0, 0);
        }
        if (store) hstore(h, slot, cat, resp);
    } else {
        resp = trial;
        if (store) hstore(h, slot, cat, add(prev, inc));
    }
    return resp;
}

/* wallHistoryResponse (:951-973) */
static v3 wall_response(v3 rate, double k, double c, double dt, v3 prev, double limit, int check_damped, int zero_at_zero,
                        hist_t* h, int slot, int cat)
{
    v3 delta = mul(rate, dt);
    v3 et = add(prev, mul(delta, k));
    v3 st = add(et, mul(rate, c));
    double tn = norm(check_damped ? st : et);
    if (tn > limit) {
        double dn = norm(delta);
        v3 lt = check_damped ? st : et;
        v3 resp = (dn > 1.0e-14 && tn > 1.0e-14) ? mul(lt, limit / tn) : (zero_at_zero ? mk(0, 0, 0) : prev);
        hstore(h, slot, cat, resp);
        return resp;
    }
    hstore(h, slot, cat, et);
    return st;
}

/* ------------------------------------------------------------------- area */
static double cross2(v2 a, v2 b) { return a.x * b.y - a.y * b.x; }
static double dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }

/* circleEdgeArea (:319-358) */
static double circle_edge_area(v2 a, v2 b, double r)
{
    v2 d = {b.x - a.x, b.y - a.y};
    double aa = dot2(d, d);
    double cuts[4] = {0.0, 1.0, 0.0, 0.0};
    int n = 2;
    if (aa > 1.0e-30) {
        double bb = 2.0 * dot2(a, d);
        double cc = dot2(a, a) - r * r;
        double disc = bb * bb - 4.0 * aa * cc;
        if (disc > 0.0) {
            double root = sqrt(disc);
            double t0 = (-bb - root) / (2.0 * aa), t1 = (-bb + root) / (2.0 * aa);
            if (t0 > 0.0 && t0 < 1.0) cuts[n++] = t0;
            if (t1 > 0.0 && t1 < 1.0) cuts[n++] = t1;
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            if (cuts[j] < cuts[i]) { double tmp = cuts[i]; cuts[i] = cuts[j]; cuts[j] = tmp; }
    double area = 0.0;
    for (int i = 0; i + 1 < n; ++i) {
        double ta = cuts[i], tb = cuts[i + 1];
        v2 u = {a.x + d.x * ta, a.y + d.y * ta};
        v2 v = {a.x + d.x * tb, a.y + d.y * tb};
        double tm = 0.5 * (ta + tb);
        v2 m = {a.x + d.x * tm, a.y + d.y * tm};
        if (dot2(m, m) <= r * r) area += 0.5 * cross2(u, v);
        else area += 0.5 * r * r * atan2(cross2(u, v), dot2(u, v));
    }
    return area;
}

/* circleTriangleArea (:360-378) */
double orc_circle_triangle_area(const double* center, const double* normal, const double* a, const double* b,
                                const double* c, double r)
{
    v3 nn = mk(normal[0], normal[1], normal[2]);
    v3 axis = fabs(nn.x) < 0.8 ? mk(1, 0, 0) : mk(0, 1, 0);
    v3 u = normalized(cross(nn, axis));
    v3 v = cross(nn, u);
    v3 ce = mk(center[0], center[1], center[2]);
    v3 ra = sub(mk(a[0], a[1], a[2]), ce), rb = sub(mk(b[0], b[1], b[2]), ce), rc = sub(mk(c[0], c[1], c[2]), ce);
    v2 pa = {dot(ra, u), dot(ra, v)}, pb = {dot(rb, u), dot(rb, v)}, pc = {dot(rc, u), dot(rc, v)};
    double area = circle_edge_area(pa, pb, r) + circle_edge_area(pb, pc, r) + circle_edge_area(pc, pa, r);
    area = fabs(area);
    return fmin(area, ORC_PI * r * r);
}

/* bodyTriangleAreaScale (:380-407) */
static double tri_area_scale(const orc* o, int comp, int tri)
{
    const double* W = o->tw + 15 * tri;
    v3 n = mk(W[12], W[13], W[14]);
    v3 a = mk(W[3], W[4], W[5]);
    v3 p = ld3(o->cpos, comp);
    double dist = dot(n, sub(p, a));
    if (dist <= 0.0) return 0.0;
    double r = o->crad[comp];
    double c2 = r * r - dist * dist;
    if (c2 <= 1.0e-30) return 0.0;
    double cr = sqrt(c2);
    v3 ce = sub(p, mul(n, dist));
    double cc[3] = {ce.x, ce.y, ce.z}, nn[3] = {n.x, n.y, n.z};
    double area = orc_circle_triangle_area(cc, nn, W + 3, W + 6, W + 9, cr);
    if (area <= 0.0) return 0.0;
    double s = fmin(1.0, area / (ORC_PI * c2));
    return s > 1.0e-12 ? s : 0.0;
}

/* ------------------------------------------------------------------- laws */
static v3 owner_omega_world(const orc* o, int i) { return rot_iv(o->quat + 4 * i, ld3(o->omg, i)); }
static v3 owner_half_omega_world(const orc* o, int i) { return rot_iv(o->quat + 4 * i, ld3(o->wh, i)); }

/* particleContact (:579-706) */
static void particle_contact(orc* o, const mech_t* m, int ci, int cj, int step, v3* fsum, v3* tsum, tls_t* tl)
{
    int i = o->cowner[ci], j = o->cowner[cj];
    if (i == j) return;
    v3 pi = ld3(o->cpos, ci), pj = ld3(o->cpos, cj);
    v3 delta = sub(pj, pi);
    double d2 = pp_distance_squared(delta);
    double ri = o->crad[ci], rj = o->crad[cj], rs = ri + rj;
    if (d2 >= rs * rs || d2 <= 1.0e-28) return;
    double d = sqrt(d2);
    double depth = rs - d;
    v3 n = mul(delta, 1.0 / d);
    v3 evi = ld3(o->cvel, ci), evj = ld3(o->cvel, cj);
    v3 erv = sub(evj, evi);
    v3 mvi = (m->dt > 0.0 && o->status[i] != -1) ? ld3(o->cvh, ci) : evi;
    v3 mvj = (m->dt > 0.0 && o->status[j] != -1) ? ld3(o->cvh, cj) : evj;
    v3 mrv = sub(mvj, mvi);
    v3 ewi = owner_omega_world(o, i), ewj = owner_omega_world(o, j);
    v3 mwi = (m->dt > 0.0 && o->status[i] != -1) ? owner_half_omega_world(o, i) : ewi;
    v3 mwj = (m->dt > 0.0 && o->status[j] != -1) ? owner_half_omega_world(o, j) : ewj;
    double mred = o->mass[i] * o->mass[j] / (o->mass[i] + o->mass[j]);
    double kS = 2.0 * m->kN / 7.0;
    double logN = log(m->epsN);
    double cN = -2.0 * logN * sqrt(m->kN * mred / (ORC_PI * ORC_PI + logN * logN));
    double logS = log(m->epsS);
    double cS = -2.0 * logS * sqrt(kS * mred / (ORC_PI * ORC_PI + logS * logS));
    double reff = ri * rj / rs;
    double brs = m->beta * reff * m->beta * reff;
    double kT = 2.0 * kS * brs, cT = 2.0 * cS * brs, kR = m->kN * brs, cR = cN * brs;
    v3 fn = add(mul(n, -m->kN * depth), mul(n, cN * dot(erv, n)));
    fn = add(fn, mul(n, m->cohesion * 4.0 * brs));
    uint64_t key = (uint64_t)(uint32_t)o->cid[cj] + 1ull;
    int slot = acquire_slot(&o->hp, ci, key, step, &tl->pover, &tl->phigh);
    if (slot < 0) return;
    double li = (ri * ri - rj * rj + d2) / (2.0 * d);
    double lj = d - li;
    v3 etv = sub(erv, mul(n, dot(erv, n)));
    etv = add(etv, mul(cross(n, ewi), li));
    etv = add(etv, mul(cross(n, ewj), lj));
    v3 mtv = sub(mrv, mul(n, dot(mrv, n)));
    mtv = add(mtv, mul(cross(n, mwi), li));
    mtv = add(mtv, mul(cross(n, mwj), lj));
    v3 old_t = transport_tangent(hload(&o->hp, slot, 1), n);
    v3 fr = limited_rates(mtv, etv, kS, cS, m->dt, old_t, m->mu * norm(fn), &o->hp, slot, 1, 1, NULL);
    v3 erw = sub(ewj, ewi), mrw = sub(mwj, mwi);
    v3 etw = mul(n, dot(erw, n)), mtw = mul(n, dot(mrw, n));
    v3 erl = sub(erw, etw), mrl = sub(mrw, mtw);
    double ms = m->beta * reff * norm(fn);
    v3 tw = limited_rates(mtw, etw, kT, cT, m->dt, transport_axial(hload(&o->hp, slot, 2), n), m->mu * m->muT * ms,
                          &o->hp, slot, 2, 1, NULL);
    v3 rl = limited_rates(mrl, erl, kR, cR, m->dt, transport_tangent(hload(&o->hp, slot, 0), n), m->muR * ms, &o->hp,
                          slot, 0, 1, NULL);
    v3 cf = add(fn, fr);
    v3 cc = add(add(tw, rl), mul(cross(n, fr), li));
    *fsum = add(*fsum, cf);
    *tsum = add(*tsum, add(cc, cross(ld3(o->coff, ci), cf)));
    tl->pcontacts++;
}

/* bodyContact (:708-853), read-only history (dt = 0, storeHistory = false) */
static void body_contact(orc* o, const mech_t* m, int comp, int tri, int hslot, v3* fsum, v3* tsum, tls_t* tl)
{
    int pi = o->cowner[comp];
    int b = o->tbody[tri];
    const double* W = o->tw + 15 * tri;
    v3 n = mk(W[12], W[13], W[14]);
    v3 a = mk(W[3], W[4], W[5]);
    v3 p = ld3(o->cpos, comp);
    double dist = dot(n, sub(p, a));
    if (dist <= 0.0) return;
    double r = o->crad[comp];
    double depth = r - dist;
    if (depth <= 0.0) return;
    double c2 = r * r - dist * dist;
    if (c2 <= 1.0e-30) return;
    double cr = sqrt(c2);
    v3 ce = sub(p, mul(n, dist));
    double cc[3] = {ce.x, ce.y, ce.z}, nn[3] = {n.x, n.y, n.z};
    double area = orc_circle_triangle_area(cc, nn, W + 3, W + 6, W + 9, cr);
    if (area <= 0.0) return;
    double as = fmin(1.0, area / (ORC_PI * c2));
    if (as <= 1.0e-12) return;
    n = mul(n, -1.0);
    v3 center = ld3(o->bc, b);
    v3 arm = sub(ce, center);
    v3 wp = owner_omega_world(o, pi);
    v3 wb = rot_iv(o->bq + 4 * b, ld3(o->bw, b));
    v3 bvel = add(ld3(o->bv, b), cross(wb, arm));
    v3 rv = sub(bvel, ld3(o->cvel, comp));
    double kS = 2.0 * m->kN / 7.0;
    double mred = o->mass[pi];
    double logN = log(m->epsN);
    double cN = -2.0 * logN * sqrt(m->kN * mred / (ORC_PI * ORC_PI + logN * logN));
    double logS = log(m->epsS);
    double cS = -2.0 * logS * sqrt(kS * mred / (ORC_PI * ORC_PI + logS * logS));
    double brs = m->beta * r * m->beta * r;
    double kT = 2.0 * kS * brs, cT = 2.0 * cS * brs, kR = m->kN * brs, cR = cN * brs;
    v3 fn = add(mul(n, -m->kN * depth), mul(n, cN * dot(rv, n)));
    fn = add(fn, mul(n, m->cohesion * 4.0 * brs));
    v3 tv = sub(rv, mul(n, dot(rv, n)));
    tv = add(tv, mul(cross(n, wp), dist));
    v3 fr = limited_rates(tv, tv, kS, cS, m->dt, transport_tangent(hload(&o->hb, hslot, 1), n), m->mu * norm(fn), &o->hb,
                          hslot, 1, 0, NULL);
    v3 rw = sub(wb, wp);
    v3 twr = mul(n, dot(rw, n));
    v3 rlr = add(sub(rw, twr), mul(cross(n, tv), 0.5 / fmax(dist, 1.0e-14)));
    double ms = m->beta * r * norm(fn);
    v3 tw = limited_rates(twr, twr, kT, cT, m->dt, transport_axial(hload(&o->hb, hslot, 2), n), m->mu * m->muT * ms, &o->hb,
                          hslot, 2, 0, NULL);
    v3 rl = limited_rates(rlr, rlr, kR, cR, m->dt, transport_tangent(hload(&o->hb, hslot, 0), n), m->muR * ms, &o->hb,
                          hslot, 0, 0, NULL);
    v3 pf = mul(add(fn, fr), as);
    v3 cm = add(tw, rl);
    v3 cpl = mul(add(cm, mul(cross(n, fr), dist)), as);
    v3 pt = add(cpl, cross(ld3(o->coff, comp), pf));
    v3 bnf = mul(fn, -as), bfr = mul(fr, -as);
    v3 bnt = mul(cross(arm, fn), -as), bft = mul(cross(arm, fr), -as);
    v3 btw = mul(tw, -as), brl = mul(rl, -as);
    v3 bt = add(add(bnt, bft), add(btw, brl));
    *fsum = add(*fsum, pf);
    *tsum = add(*tsum, pt);
    if (o->fbodyp) {
        double* d = o->fbodyp + ((size_t)b * o->n + pi) * 6;
        d[0] += pf.x; d[1] += pf.y; d[2] += pf.z; d[3] += pt.x; d[4] += pt.y; d[5] += pt.z;
    }
    if (o->fbodyd) {
        double* d = o->fbodyd + ((size_t)b * o->n + pi) * 19;
        v3 vals[6] = {bnf, bfr, bnt, bft, btw, brl};
        for (int g = 0; g < 6; ++g) { d[3 * g] += vals[g].x; d[3 * g + 1] += vals[g].y; d[3 * g + 2] += vals[g].z; }
        if (d[18] < depth) d[18] = depth;
    }
    double* R = tl->bres + 6 * b;
    R[0] += bnf.x + bfr.x; R[1] += bnf.y + bfr.y; R[2] += bnf.z + bfr.z;
    R[3] += bt.x; R[4] += bt.y; R[5] += bt.z;
    tl->bcontacts++;
    if (depth > tl->bmaxdepth) tl->bmaxdepth = depth;
    tl->bfz += bnf.z + bfr.z;
}

/* advanceBodyManifoldHistory (:855-949) */
static int manifold_history(orc* o, const mech_t* m, int comp, int b, int step, v3 n, v3 ce, double dist, int* slide,
                            int* twist, tls_t* tl)
{
    *slide = 0; *twist = 0;
    int pi = o->cowner[comp];
    uint64_t key = (uint64_t)(b + 1);
    int slot = acquire_slot(&o->hb, comp, key, step, &tl->bover, &tl->bhigh);
    if (slot < 0) return -1;
    v3 center = ld3(o->bc, b);
    v3 arm = sub(ce, center);
    v3 ewp = owner_omega_world(o, pi);
    int dyn = m->dt > 0.0 && o->status[pi] != -1;
    v3 mwp = dyn ? owner_half_omega_world(o, pi) : ewp;
    v3 wb = rot_iv(o->bq + 4 * b, ld3(o->bw, b));
    v3 bvel = add(ld3(o->bv, b), cross(wb, arm));
    v3 evp = ld3(o->cvel, comp);
    v3 mvp = dyn ? ld3(o->cvh, comp) : evp;
    v3 erv = sub(bvel, evp), mrv = sub(bvel, mvp);
    double kS = 2.0 * m->kN / 7.0;
    double mred = o->mass[pi];
    double logN = log(m->epsN);
    double cN = -2.0 * logN * sqrt(m->kN * mred / (ORC_PI * ORC_PI + logN * logN));
    double logS = log(m->epsS);
    double cS = -2.0 * logS * sqrt(kS * mred / (ORC_PI * ORC_PI + logS * logS));
    double r = o->crad[comp];
    double brs = m->beta * r * m->beta * r;
    double kT = 2.0 * kS * brs, cT = 2.0 * cS * brs, kR = m->kN * brs, cR = cN * brs;
    double depth = r - dist;
    v3 fn = add(mul(n, -m->kN * depth), mul(n, cN * dot(erv, n)));
    fn = add(fn, mul(n, m->cohesion * 4.0 * brs));
    v3 tv = sub(mrv, mul(n, dot(mrv, n)));
    tv = add(tv, mul(cross(n, mwp), dist));
    limited_rates(tv, tv, kS, cS, m->dt, transport_tangent(hload(&o->hb, slot, 1), n), m->mu * norm(fn), &o->hb, slot, 1,
                  1, slide);
    v3 rw = sub(wb, mwp);
    v3 twr = mul(n, dot(rw, n));
    v3 rlr = add(sub(rw, twr), mul(cross(n, tv), 0.5 / fmax(dist, 1.0e-14)));
    double ms = m->beta * r * norm(fn);
    limited_rates(twr, twr, kT, cT, m->dt, transport_axial(hload(&o->hb, slot, 2), n), m->mu * m->muT * ms, &o->hb, slot, 2,
                  1, twist);
    limited_rates(rlr, rlr, kR, cR, m->dt, transport_tangent(hload(&o->hb, slot, 0), n), m->muR * ms, &o->hb, slot, 0, 1,
                  NULL);
    return slot;
}

/* wallContact (:975-1063) */
static void wall_contact(orc* o, const mech_t* m, int comp, int w, int step, v3* fsum, v3* tsum, tls_t* tl)
{
    int pi = o->cowner[comp];
    v3 out = ld3(o->wn, w);
    v3 n = mul(out, -1.0);
    v3 org = ld3(o->wo, w);
    v3 p = ld3(o->cpos, comp);
    double dist = dot(sub(p, org), out);
    double depth = o->crad[comp] - dist;
    if (depth <= 0.0) return;
    uint64_t key = (uint64_t)w + 1ull;
    int slot = acquire_slot(&o->hw, comp, key, step, &tl->bover, &tl->bhigh);
    if (slot < 0) return;
    double r = o->crad[comp];
    double lever = r - depth;
    v3 vel = ld3(o->cvel, comp);
    v3 om = owner_omega_world(o, pi);
    v3 rv = mul(vel, -1.0);
    v3 tv = sub(rv, mul(n, dot(rv, n)));
    tv = add(tv, mul(cross(n, om), lever));
    v3 rw = mul(om, -1.0);
    v3 twr = mul(n, dot(rw, n));
    v3 rlr = sub(rw, twr);
    if (fabs(lever) > 1.0e-30) rlr = add(rlr, mul(cross(n, tv), 0.5 / lever));
    double kS = 2.0 * m->kN / 7.0;
    double logN = log(m->epsN);
    double cN = -2.0 * logN * sqrt(m->kN * o->mass[pi] / (ORC_PI * ORC_PI + logN * logN));
    double logS = log(m->epsS);
    double cS = -2.0 * logS * sqrt(kS * o->mass[pi] / (ORC_PI * ORC_PI + logS * logS));
    double brs = m->beta * r * m->beta * r;
    double kT = 2.0 * kS * brs, cT = 2.0 * cS * brs, kR = m->kN * brs, cR = cN * brs;
    v3 en = mul(n, -m->kN * depth);
    v3 dn = mul(n, cN * dot(rv, n));
    v3 fn = add(en, dn);
    double flim = m->mu * norm(fn);
    double ms = m->beta * r * norm(fn);
    v3 fr = wall_response(tv, kS, cS, m->dt, transport_tangent(hload(&o->hw, slot, 1), n), flim, 0, 0, &o->hw, slot, 1);
    v3 tw = wall_response(twr, kT, cT, m->dt, transport_axial(hload(&o->hw, slot, 2), n), m->mu * m->muT * ms, 0, 1, &o->hw,
                          slot, 2);
    v3 rl = wall_response(rlr, kR, cR, m->dt, transport_tangent(hload(&o->hw, slot, 0), n), m->muR * ms, 1, 1, &o->hw,
                          slot, 0);
    v3 cf = add(fn, fr);
    v3 cc = add(add(tw, rl), mul(cross(n, fr), lever));
    *fsum = add(*fsum, cf);
    *tsum = add(*tsum, add(cc, cross(ld3(o->coff, comp), cf)));
}

/* manifold sums over the component's own triangle-grid cell (:1154-1183) */
static double manifold_sums(const orc* o, int comp, int b, int begin, int end, v3* wn, v3* wc, double* wd)
{
    v3 p = ld3(o->cpos, comp);
    double tot = 0.0;
    *wn = mk(0, 0, 0); *wc = mk(0, 0, 0); *wd = 0.0;
    for (int e = begin; e < end; ++e) {
        int tri = o->tid[e];
        if (o->tbody[tri] != b) continue;
        double as = tri_area_scale(o, comp, tri);
        if (as <= 0.0) continue;
        const double* W = o->tw + 15 * tri;
        v3 out = mk(W[12], W[13], W[14]);
        v3 a = mk(W[3], W[4], W[5]);
        double dist = dot(out, sub(p, a));
        v3 ce = sub(p, mul(out, dist));
        tot += as;
        *wn = add(*wn, mul(out, -as));
        *wc = add(*wc, mul(ce, as));
        *wd += dist * as;
    }
    return tot;
}

/* computeContactsKernel (:1065-1221), one owner */
static void contacts_owner(orc* o, int i, const mech_t* pm, const mech_t* bm, const mech_t* wm, int step, tls_t* tl)
{
    v3 cF = mk(0, 0, 0), cT = mk(0, 0, 0), fF = mk(0, 0, 0), wF = mk(0, 0, 0), wT = mk(0, 0, 0), bF = mk(0, 0, 0),
       bT = mk(0, 0, 0);
    if (o->grav) fF = mk(o->mass[i] * o->g[0], o->mass[i] * o->g[1], o->mass[i] * o->g[2]);
    if (o->ugrav) {
        v3 pi = ld3(o->pos, i);
        for (int j = 0; j < o->n; ++j) {
            if (j == i) continue;
            v3 dl = sub(pi, ld3(o->pos, j));
            double d2 = dot(dl, dl);
            if (d2 > 1.0e-28) fF = add(fF, mul(dl, ORC_G * o->mass[i] * o->mass[j] / (d2 * sqrt(d2))));
        }
    }
    for (int comp = o->ostart[i]; comp < o->ostart[i + 1]; ++comp) {
        expire(&o->hp, comp, step);
        expire(&o->hw, comp, step);
        expire(&o->hb, comp, step);
        for (int w = 0; w < o->nw; ++w) wall_contact(o, wm, comp, w, step, &wF, &wT, tl);
        v3 p = ld3(o->cpos, comp);
        int ix = (int)floor(p.x * o->inv_mesh), iy = (int)floor(p.y * o->inv_mesh), iz = (int)floor(p.z * o->inv_mesh);
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    uint64_t key = pack_cell(ix + dx, iy + dy, iz + dz);
                    int b = lower_bound_u64(o->skey, o->nc, key), e = upper_bound_u64(o->skey, o->nc, key);
                    for (int k = b; k < e; ++k) {
                        int other = o->sid[k];
                        if (o->cowner[other] != i) particle_contact(o, pm, comp, other, step, &cF, &cT, tl);
                    }
                }
        if (o->nt <= 0 || o->tentries <= 0) continue;
        uint64_t key = pack_cell(ix, iy, iz);
        int tb = lower_bound_u64(o->tkey, o->tentries, key), te = upper_bound_u64(o->tkey, o->tentries, key);
        for (int b = 0; b < o->nb; ++b) {
            v3 wn, wc;
            double wd;
            double tot = manifold_sums(o, comp, b, tb, te, &wn, &wc, &wd);
            if (tot <= 0.0) continue;
            v3 mn = normalized(wn);
            v3 mc = mul(wc, 1.0 / tot);
            double md = wd / tot;
            int slide = 0, twist = 0;
            int hs = manifold_history(o, bm, comp, b, step, mn, mc, md, &slide, &twist, tl);
            if (hs < 0) continue;
            o->regime_state[(size_t)b * o->nc + comp] = 1 | (slide ? 2 : 0) | (twist ? 4 : 0);
            mech_t ro = *bm;
            ro.dt = 0.0;
            for (int e = tb; e < te; ++e) {
                int tri = o->tid[e];
                if (o->tbody[tri] != b) continue;
                body_contact(o, &ro, comp, tri, hs, &bF, &bT, tl);
            }
        }
    }
    double* c6 = o->fcontact + 6 * (size_t)i;
    c6[0] += cF.x; c6[1] += cF.y; c6[2] += cF.z; c6[3] += cT.x; c6[4] += cT.y; c6[5] += cT.z;
    double* f6 = o->ffield + 6 * (size_t)i;
    f6[0] += fF.x; f6[1] += fF.y; f6[2] += fF.z;
    double* w6 = o->fwall + 6 * (size_t)i;
    w6[0] += wF.x; w6[1] += wF.y; w6[2] += wF.z; w6[3] += wT.x; w6[4] += wT.y; w6[5] += wT.z;
    v3 TF = add(add(cF, fF), add(wF, bF));
    v3 TT = add(cT, add(wT, bT));
    double* t6 = o->ftotal + 6 * (size_t)i;
    t6[0] += TF.x; t6[1] += TF.y; t6[2] += TF.z; t6[3] += TT.x; t6[4] += TT.y; t6[5] += TT.z;
    st3(o->f, i, TF);
    st3(o->t, i, TT);
}

/* observeBodyMicrostateKernel (:1226-1356), one (body, component) */
static void observe_microstate(orc* o, const mech_t* m, int b, int comp, int step)
{
    size_t index = (size_t)b * o->nc + comp;
    if ((o->regime_state[index] & 1) == 0) return;
    v3 p = ld3(o->cpos, comp);
    int ix = (int)floor(p.x * o->inv_mesh), iy = (int)floor(p.y * o->inv_mesh), iz = (int)floor(p.z * o->inv_mesh);
    uint64_t key = pack_cell(ix, iy, iz);
    int tb = lower_bound_u64(o->tkey, o->tentries, key), te = upper_bound_u64(o->tkey, o->tentries, key);
    v3 wn, wc;
    double wd;
    double tot = manifold_sums(o, comp, b, tb, te, &wn, &wc, &wd);
    if (tot <= 0.0) return;
    uint64_t hkey = (uint64_t)(b + 1);
    int hslot = -1;
    for (int s = 0; s < BSLOTS; ++s) {
        int idx = comp * BSLOTS + s;
        if (o->hb.keys[idx] == hkey && o->hb.last[idx] == step) { hslot = idx; break; }
    }
    if (hslot < 0) return;
    v3 n = normalized(wn);
    v3 ce = mul(wc, 1.0 / tot);
    double dist = wd / tot;
    int pi = o->cowner[comp];
    v3 center = ld3(o->bc, b);
    v3 arm = sub(ce, center);
    v3 wb = rot_iv(o->bq + 4 * b, ld3(o->bw, b));
    v3 bvel = add(ld3(o->bv, b), cross(wb, arm));
    v3 rv = sub(bvel, ld3(o->cvel, comp));
    double mred = o->mass[pi];
    double logN = log(m->epsN);
    double cN = -2.0 * logN * sqrt(m->kN * mred / (ORC_PI * ORC_PI + logN * logN));
    double r = o->crad[comp];
    double brs = m->beta * r * m->beta * r;
    double depth = r - dist;
    v3 fn = add(mul(n, -m->kN * depth), mul(n, cN * dot(rv, n)));
    fn = add(fn, mul(n, m->cohesion * 4.0 * brs));
    double fnn = norm(fn);
    double ms = m->beta * r * fnn;
    double tl = m->mu * fnn;
    double twl = m->mu * m->muT * ms;
    v3 th = hload(&o->hb, hslot, 1), twh = hload(&o->hb, hslot, 2);
    v3 az = rot_iv(o->bq + 4 * b, mk(0, 0, 1));
    v3 radial = sub(arm, mul(az, dot(arm, az)));
    double tu = tl > 1.0e-30 ? fmin(1.0, norm(th) / tl) : 0.0;
    double twu = twl > 1.0e-30 ? fmin(1.0, norm(twh) / twl) : 0.0;
    v3 btw = mul(twh, -tot), bnl = mul(fn, -tot), bth = mul(th, -tot);
    v3 btt = cross(arm, bth);
    double* ms22 = o->micro_state + index * NMICRO;
    ms22[0] = fnn * tot; ms22[1] = fnn * r * tot; ms22[2] = fnn * norm(radial) * tot;
    ms22[3] = btw.x; ms22[4] = btw.y; ms22[5] = btw.z;
    ms22[6] = norm(twh) * tot; ms22[7] = twl * tot; ms22[8] = norm(th) * tot; ms22[9] = tl * tot;
    ms22[10] = twu * tot; ms22[11] = tu * tot; ms22[12] = tot;
    ms22[13] = bnl.x; ms22[14] = bnl.y; ms22[15] = bnl.z;
    ms22[16] = bth.x; ms22[17] = bth.y; ms22[18] = bth.z;
    ms22[19] = btt.x; ms22[20] = btt.y; ms22[21] = btt.z;
}

/* accumulateBodyRegimeKernel (:530-567), sequential */
static void accumulate_regime(orc* o, int interval)
{
    for (int b = 0; b < o->nb; ++b)
        for (int c = 0; c < o->nc; ++c) {
            size_t index = (size_t)b * o->nc + c;
            int st = o->regime_state[index];
            if ((st & 1) == 0) continue;
            int sl = (st & 2) != 0, tw = (st & 4) != 0;
            int prim = tw ? 3 : (sl ? 2 : 1);
            unsigned long long* R = o->reg_inst + b * NREG;
            R[0]++; R[prim]++; if (sl) R[4]++; if (tw) R[5]++; if (sl && tw) R[6]++;
            for (int f = 0; f < NMICRO; ++f) o->micro_inst[b * NMICRO + f] += o->micro_state[index * NMICRO + f];
            if (!interval) continue;
            R = o->reg_int + b * NREG;
            R[0]++; R[prim]++; if (sl) R[4]++; if (tw) R[5]++; if (sl && tw) R[6]++;
            for (int f = 0; f < NMICRO; ++f) o->micro_int[b * NMICRO + f] += o->micro_state[index * NMICRO + f];
        }
}

/* accelerationKernel (src/cuda/cuda_particle_backend.cu:71-101) */
static void acceleration(orc* o)
{
    for (int i = 0; i < o->n; ++i) {
        double m = o->mass[i];
        o->acc[3 * i] = o->f[3 * i] / m; o->acc[3 * i + 1] = o->f[3 * i + 1] / m; o->acc[3 * i + 2] = o->f[3 * i + 2] / m;
        double qw = o->quat[4 * i], qx = o->quat[4 * i + 1], qy = o->quat[4 * i + 2], qz = o->quat[4 * i + 3];
        double Tx = o->t[3 * i], Ty = o->t[3 * i + 1], Tz = o->t[3 * i + 2];
        double tx = (1.0 - 2.0 * (qy * qy + qz * qz)) * Tx + 2.0 * (qx * qy + qw * qz) * Ty + 2.0 * (qx * qz - qw * qy) * Tz;
        double ty = 2.0 * (qx * qy - qw * qz) * Tx + (1.0 - 2.0 * (qx * qx + qz * qz)) * Ty + 2.0 * (qy * qz + qw * qx) * Tz;
        double tz = 2.0 * (qx * qz + qw * qy) * Tx + 2.0 * (qy * qz - qw * qx) * Ty + (1.0 - 2.0 * (qx * qx + qy * qy)) * Tz;
        double wx = o->omg[3 * i], wy = o->omg[3 * i + 1], wz = o->omg[3 * i + 2];
        double Ix = o->inertia[3 * i], Iy = o->inertia[3 * i + 1], Iz = o->inertia[3 * i + 2];
        o->aacc[3 * i] = (tx - (Iz - Iy) * wz * wy) / Ix;
        o->aacc[3 * i + 1] = (ty - (Ix - Iz) * wx * wz) / Iy;
        o->aacc[3 * i + 2] = (tz - (Iy - Ix) * wy * wx) / Iz;
    }
}

/* CudaDemSolver::computeForces (src/cuda_backend_cuda.cu:383-524) */
int orc_compute_forces(orc* o, const double* bc, const double* bq, const double* bv, const double* bw, double* body_forces,
                       int diag)
{
    int nb = o->nb;
    if (nb > 0 && bc) {
        memcpy(o->bc, bc, 3 * nb * sizeof(double)); memcpy(o->bq, bq, 4 * nb * sizeof(double));
        memcpy(o->bv, bv, 3 * nb * sizeof(double)); memcpy(o->bw, bw, 3 * nb * sizeof(double));
    }
    if (nb > 0) transform_triangles(o);
    update_components(o);
    int rc = build_particle_grid(o);
    if (rc) return rc;
    if (o->nt > 0) { rc = build_triangle_grid(o); if (rc) return rc; }
    /* clearForcesKernel (src/cuda/cuda_contact_backend.cu:478-528) */
    size_t n6 = 6 * (size_t)o->n;
    memset(o->fcontact, 0, n6 * sizeof(double)); memset(o->ffield, 0, n6 * sizeof(double));
    memset(o->fwall, 0, n6 * sizeof(double)); memset(o->ftotal, 0, n6 * sizeof(double));
    if (o->fbodyp) memset(o->fbodyp, 0, (size_t)nb * n6 * sizeof(double));
    if (o->fbodyd) memset(o->fbodyd, 0, (size_t)nb * o->n * 19 * sizeof(double));
    if (nb > 0) {
        memset(o->reg_inst, 0, nb * NREG * sizeof(unsigned long long));
        memset(o->regime_state, 0, (size_t)nb * o->nc * sizeof(int));
        memset(o->micro_state, 0, (size_t)nb * o->nc * NMICRO * sizeof(double));
        memset(o->micro_inst, 0, nb * NMICRO * sizeof(double));
    }
    memset(o->bres, 0, (nb > 0 ? nb : 1) * 6 * sizeof(double));
    o->pcontacts = 0; o->bcontacts = 0; o->phigh = 0; o->bhigh = 0; o->bmaxdepth = 0.0; o->bfz = 0.0;

    const int step = o->step_index++;
    mech_t pm = o->pp, bm = o->pt, wm = o->pw;
    if (step == 0) { pm.dt = 0.0; bm.dt = 0.0; wm.dt = 0.0; }
    int nth = o->nthreads;
    tls_t* tls = zalloc(nth * sizeof(tls_t));
    for (int k = 0; k < nth; ++k) tls[k].bres = zalloc((nb > 0 ? nb : 1) * 6 * sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nth)
#endif
    for (int i = 0; i < o->n; ++i) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        contacts_owner(o, i, &pm, &bm, &wm, step, &tls[tid]);
    }
    for (int k = 0; k < nth; ++k) {
        o->pcontacts += tls[k].pcontacts; o->bcontacts += tls[k].bcontacts;
        o->pover += tls[k].pover; o->bover += tls[k].bover;
        if (tls[k].phigh > o->phigh) o->phigh = tls[k].phigh;
        if (tls[k].bhigh > o->bhigh) o->bhigh = tls[k].bhigh;
        if (tls[k].bmaxdepth > o->bmaxdepth) o->bmaxdepth = tls[k].bmaxdepth;
        o->bfz += tls[k].bfz;
        for (int q = 0; q < nb * 6; ++q) o->bres[q] += tls[k].bres[q];
        free(tls[k].bres);
    }
    free(tls);
    if (nb > 0) {
        for (int b = 0; b < nb; ++b)
            for (int c = 0; c < o->nc; ++c) observe_microstate(o, &bm, b, c, step);
        accumulate_regime(o, bm.dt > 0.0);
        if (bm.dt > 0.0) o->reg_native_steps++;
    }
    acceleration(o);
    if (diag) {
        dem_step_stats* s = &o->stats;
        memset(s, 0, sizeof *s);
        s->particle_contacts = o->pcontacts; s->body_contacts = o->bcontacts;
        s->body_max_depth = o->bmaxdepth; s->body_contact_fz = o->bfz;
        s->particle_history_overflows = o->pover; s->body_history_overflows = o->bover;
        s->particle_history_high_water = o->phigh; s->body_history_high_water = o->bhigh;
        s->triangle_grid_overflows = o->tgover;
        s->body_regime_interval_native_steps = o->reg_native_steps;
        /* download the counters and sums, then reset the interval ones
         * (src/cuda_backend_cuda.cu:431-482) */
        if (nb > 0) {
            memcpy(o->diag_reg_inst, o->reg_inst, nb * NREG * sizeof(unsigned long long));
            memcpy(o->diag_reg_int, o->reg_int, nb * NREG * sizeof(unsigned long long));
            memcpy(o->diag_micro_inst, o->micro_inst, nb * NMICRO * sizeof(double));
            memcpy(o->diag_micro_int, o->micro_int, nb * NMICRO * sizeof(double));
            memset(o->reg_int, 0, nb * NREG * sizeof(unsigned long long));
            memset(o->micro_int, 0, nb * NMICRO * sizeof(double));
            o->reg_native_steps = 0;
        }
        if (o->pover) { set_error("particle contact-history capacity exceeded"); return DEM_ERR_CAPACITY; }
        if (o->bover) { set_error("wall/body contact-history capacity exceeded"); return DEM_ERR_CAPACITY; }
    }
    if (body_forces && nb > 0) {
        for (int b = 0; b < nb; ++b) {
            for (int k = 0; k < 6; ++k) body_forces[6 * b + k] = o->bres[6 * b + k];
            if (o->grav) {
                body_forces[6 * b] += o->g[0] * o->bmass[b];
                body_forces[6 * b + 1] += o->g[1] * o->bmass[b];
                body_forces[6 * b + 2] += o->g[2] * o->bmass[b];
            }
        }
    }
    return DEM_OK;
}

/* The regime counters and microstate sums of the last diagnostic
 * evaluation, as CudaStepStats carries them (src/cuda_backend_cuda.cu:431-482). */
void orc_body_diagnostics(orc* o, unsigned long long* ri, unsigned long long* rv, double* mi, double* mv)
{
    int nb = o->nb;
    if (nb <= 0) return;
    if (ri) memcpy(ri, o->diag_reg_inst, nb * NREG * sizeof(unsigned long long));
    if (rv) memcpy(rv, o->diag_reg_int, nb * NREG * sizeof(unsigned long long));
    if (mi) memcpy(mi, o->diag_micro_inst, nb * NMICRO * sizeof(double));
    if (mv) memcpy(mv, o->diag_micro_int, nb * NMICRO * sizeof(double));
}

/* ---------------------------------------------------------------- leapfrog */
/* quatDerivative / normalizeQuat (src/cuda/cuda_particle_backend.cu:149-183) */
static void quat_derivative(const double* q, double wx, double wy, double wz, double* d)
{
    d[0] = 0.5 * (-q[1] * wx - q[2] * wy - q[3] * wz);
    d[1] = 0.5 * (q[0] * wx + q[2] * wz - q[3] * wy);
    d[2] = 0.5 * (q[0] * wy - q[1] * wz + q[3] * wx);
    d[3] = 0.5 * (q[0] * wz + q[1] * wy - q[2] * wx);
}
static void normalize_quat(double* q)
{
    double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (n2 <= 1.0e-24) { q[0] = 1.0; q[1] = q[2] = q[3] = 0.0; return; }
    double inv = 1.0 / sqrt(n2);
    q[0] *= inv; q[1] *= inv; q[2] *= inv; q[3] *= inv;
}

/* initializeLeapfrogKernel (:185-210) */
int orc_leapfrog_init(orc* o, double h)
{
    for (int i = 0; i < o->n; ++i) {
        for (int a = 0; a < 3; ++a) {
            o->vh[3 * i + a] = o->vel[3 * i + a] + o->acc[3 * i + a] * h;
            o->wh[3 * i + a] = o->omg[3 * i + a] + o->aacc[3 * i + a] * h;
        }
        double q[4] = {o->quat[4 * i], o->quat[4 * i + 1], o->quat[4 * i + 2], o->quat[4 * i + 3]}, d[4];
        quat_derivative(q, o->omg[3 * i], o->omg[3 * i + 1], o->omg[3 * i + 2], d);
        for (int k = 0; k < 4; ++k) q[k] += d[k] * h;
        normalize_quat(q);
        quat_derivative(q, o->wh[3 * i], o->wh[3 * i + 1], o->wh[3 * i + 2], o->hdq + 4 * i);
    }
    return DEM_OK;
}

/* advancePositionKernel (:212-237) */
int orc_advance(orc* o, double dt)
{
    for (int i = 0; i < o->n; ++i) {
        if (o->status[i] == -1) continue;
        for (int a = 0; a < 3; ++a) o->pos[3 * i + a] += o->vh[3 * i + a] * dt;
        for (int k = 0; k < 4; ++k) o->quat[4 * i + k] += o->hdq[4 * i + k] * dt;
        normalize_quat(o->quat + 4 * i);
        for (int a = 0; a < 3; ++a) {
            o->vel[3 * i + a] = o->vh[3 * i + a] + o->acc[3 * i + a] * (0.5 * dt);
            o->omg[3 * i + a] = o->wh[3 * i + a] + o->aacc[3 * i + a] * (0.5 * dt);
        }
    }
    return DEM_OK;
}

/* advanceHalfVelocityKernel (:239-265) */
int orc_finish(orc* o, double dt)
{
    const double h = 0.5 * dt;
    for (int i = 0; i < o->n; ++i) {
        for (int a = 0; a < 3; ++a) {
            o->vh[3 * i + a] += o->acc[3 * i + a] * dt;
            o->wh[3 * i + a] += o->aacc[3 * i + a] * dt;
        }
        double q[4] = {o->quat[4 * i], o->quat[4 * i + 1], o->quat[4 * i + 2], o->quat[4 * i + 3]}, d[4];
        quat_derivative(q, o->omg[3 * i], o->omg[3 * i + 1], o->omg[3 * i + 2], d);
        for (int k = 0; k < 4; ++k) q[k] += d[k] * h;
        normalize_quat(q);
        quat_derivative(q, o->wh[3 * i], o->wh[3 * i + 1], o->wh[3 * i + 2], o->hdq + 4 * i);
    }
    return DEM_OK;
}

/* ----------------------------------------------------------- host MBD step */
/* gama (src/matrixtrans.cpp:87-96) */
static void gama(const double* q, const double* w, double* d)
{
    d[0] = 0.5 * (-q[1] * w[0] - q[2] * w[1] - q[3] * w[2]);
    d[1] = 0.5 * (q[0] * w[0] + q[2] * w[2] - q[3] * w[1]);
    d[2] = 0.5 * (q[0] * w[1] - q[1] * w[2] + q[3] * w[0]);
    d[3] = 0.5 * (q[0] * w[2] + q[1] * w[1] - q[2] * w[0]);
}
/* vector4d::normalize (include/matrixtrans.h:208-216) */
static void normalize4(double* q)
{
    double len = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    if (len > 1e-10) { double s = 1.0 / len; q[0] *= s; q[1] *= s; q[2] *= s; q[3] *= s; }
    else q[0] = q[1] = q[2] = q[3] = 0.0;
}
/* DynEqnBodySet (src/dyneq.cpp:97-130) with Quat2DCM (src/matrixtrans.cpp:36-63) */
static void dyn_eqn_bodies(orc* o, const double* F, double* ddu)
{
    for (int b = 0; b < o->nb; ++b) {
        double* d = ddu + 6 * b;
        if (o->bstate[b] != 0) { for (int k = 0; k < 6; ++k) d[k] = 0.0; continue; }
        for (int k = 0; k < 3; ++k) d[k] = F[6 * b + k] / o->bmass[b];
        const double* q = o->bq + 4 * b;
        double qq[10] = {q[0] * q[0], q[1] * q[1], q[2] * q[2], q[3] * q[3], 2.0 * q[0] * q[1], 2.0 * q[0] * q[2],
                         2.0 * q[0] * q[3], 2.0 * q[1] * q[2], 2.0 * q[1] * q[3], 2.0 * q[2] * q[3]};
        double M[9] = {qq[0] + qq[1] - qq[2] - qq[3], qq[7] + qq[6], qq[8] - qq[5],
                       qq[7] - qq[6], qq[0] - qq[1] + qq[2] - qq[3], qq[9] + qq[4],
                       qq[8] + qq[5], qq[9] - qq[4], qq[0] - qq[1] - qq[2] + qq[3]};
        double T[3] = {F[6 * b + 3], F[6 * b + 4], F[6 * b + 5]};
        double t[3];
        for (int r = 0; r < 3; ++r) t[r] = M[3 * r] * T[0] + M[3 * r + 1] * T[1] + M[3 * r + 2] * T[2];
        const double* I = o->binertia + 9 * b;
        const double* w = o->bw + 3 * b;
        d[3] = (t[0] - (I[8] - I[4]) * w[2] * w[1]) / I[0];
        d[4] = (t[1] - (I[0] - I[8]) * w[0] * w[2]) / I[4];
        d[5] = (t[2] - (I[4] - I[0]) * w[1] * w[0]) / I[8];
    }
}

static void body_half_update(orc* o, int first, double dt, double half)
{
    double* ddu = zalloc(6 * o->nb * sizeof(double));
    dyn_eqn_bodies(o, o->bloads, ddu);
    for (int b = 0; b < o->nb; ++b) {
        double* hv = o->bhalf_v + 3 * b, *hw = o->bhalf_w + 3 * b, *acc = o->bacc + 3 * b, *dom = o->bdomg + 3 * b;
        double* V = o->bv + 3 * b, *Wb = o->bw + 3 * b;
        for (int a = 0; a < 3; ++a) { acc[a] = ddu[6 * b + a]; dom[a] = ddu[6 * b + 3 + a]; }
        int st = o->bstate[b];
        if (st == 0) {
            for (int a = 0; a < 3; ++a) {
                if (first) { hv[a] = V[a] + acc[a] * half; hw[a] = Wb[a] + dom[a] * half; }
                else { hv[a] += acc[a] * dt; hw[a] += dom[a] * dt; }
            }
        } else if (st == 1) {
            for (int a = 0; a < 3; ++a) {
                acc[a] = 0.0; dom[a] = 0.0; hv[a] = 0.0; hw[a] = 0.0;
                if (!first) { V[a] = 0.0; Wb[a] = 0.0; }
            }
        } else {
            for (int a = 0; a < 3; ++a) { if (first) { acc[a] = 0.0; dom[a] = 0.0; } hv[a] = V[a]; hw[a] = Wb[a]; }
        }
        double d[4], q[4];
        gama(o->bq + 4 * b, Wb, d);
        for (int k = 0; k < 4; ++k) q[k] = o->bq[4 * b + k] + d[k] * half;
        normalize4(q);
        memcpy(o->bhalf_q + 4 * b, q, 4 * sizeof(double));
        gama(q, hw, o->bhalf_dq + 4 * b);
    }
    free(ddu);
}

/* IntegrateDem / IntegrateDemMultiBody (src/cuda_simulation_integrator.cpp:
 * 245-446) without output frames or a prescribed-motion schedule. */
int orc_run(orc* o, int steps, double dt)
{
    const double half = 0.5 * dt;
    int nb = o->nb;
    int rc;
    if (!o->started) {
        rc = orc_compute_forces(o, NULL, NULL, NULL, NULL, nb > 0 ? o->bloads : NULL, 1);
        if (rc) return rc;
        if (!o->restored_leapfrog) orc_leapfrog_init(o, half);
        if (nb > 0) body_half_update(o, 1, dt, half);
        o->started = 1;
    }
    for (int s = 0; s < steps; ++s) {
        orc_advance(o, dt);
        for (int b = 0; b < nb; ++b) {
            if (o->bstate[b] == 1) continue;
            for (int a = 0; a < 3; ++a) o->bc[3 * b + a] += o->bhalf_v[3 * b + a] * dt;
            double q[4];
            for (int k = 0; k < 4; ++k) q[k] = o->bq[4 * b + k] + o->bhalf_dq[4 * b + k] * dt;
            normalize4(q);
            memcpy(o->bq + 4 * b, q, sizeof q);
            for (int a = 0; a < 3; ++a) {
                o->bv[3 * b + a] = o->bhalf_v[3 * b + a] + o->bacc[3 * b + a] * half;
                o->bw[3 * b + a] = o->bhalf_w[3 * b + a] + o->bdomg[3 * b + a] * half;
            }
        }
        rc = orc_compute_forces(o, NULL, NULL, NULL, NULL, nb > 0 ? o->bloads : NULL, s == steps - 1);
        if (rc) return rc;
        orc_finish(o, dt);
        if (nb > 0) body_half_update(o, 0, dt, half);
        o->drv_step++;
    }
    return DEM_OK;
}

/* ---------------------------------------------------------------- accessors */
void orc_counts(const orc* o, int* out)
{
    out[0] = o->n; out[1] = o->nc; out[2] = o->nb; out[3] = o->nt; out[4] = o->nw; out[5] = o->tentries;
}
void orc_get_state(const orc* o, double* pos, double* vel, double* omg, double* quat)
{
    if (pos) memcpy(pos, o->pos, 3 * o->n * sizeof(double));
    if (vel) memcpy(vel, o->vel, 3 * o->n * sizeof(double));
    if (omg) memcpy(omg, o->omg, 3 * o->n * sizeof(double));
    if (quat) memcpy(quat, o->quat, 4 * o->n * sizeof(double));
}
void orc_set_state(orc* o, const double* pos, const double* vel, const double* omg, const double* quat)
{
    if (pos) memcpy(o->pos, pos, 3 * o->n * sizeof(double));
    if (vel) memcpy(o->vel, vel, 3 * o->n * sizeof(double));
    if (omg) memcpy(o->omg, omg, 3 * o->n * sizeof(double));
    if (quat) memcpy(o->quat, quat, 4 * o->n * sizeof(double));
}
void orc_get_half(const orc* o, double* vh, double* wh, double* hdq, double* acc, double* aacc)
{
    if (vh) memcpy(vh, o->vh, 3 * o->n * sizeof(double));
    if (wh) memcpy(wh, o->wh, 3 * o->n * sizeof(double));
    if (hdq) memcpy(hdq, o->hdq, 4 * o->n * sizeof(double));
    if (acc) memcpy(acc, o->acc, 3 * o->n * sizeof(double));
    if (aacc) memcpy(aacc, o->aacc, 3 * o->n * sizeof(double));
}
void orc_get_forces(const orc* o, double* c, double* f, double* w, double* t, double* bp, double* bd)
{
    size_t n6 = 6 * (size_t)o->n;
    if (c) memcpy(c, o->fcontact, n6 * sizeof(double));
    if (f) memcpy(f, o->ffield, n6 * sizeof(double));
    if (w) memcpy(w, o->fwall, n6 * sizeof(double));
    if (t) memcpy(t, o->ftotal, n6 * sizeof(double));
    if (bp && o->fbodyp) memcpy(bp, o->fbodyp, (size_t)o->nb * n6 * sizeof(double));
    if (bd && o->fbodyd) memcpy(bd, o->fbodyd, (size_t)o->nb * o->n * 19 * sizeof(double));
}
void orc_get_body_result(const orc* o, double* res) { if (o->nb > 0) memcpy(res, o->bres, 6 * o->nb * sizeof(double)); }
void orc_get_bodies(const orc* o, double* c, double* q, double* v, double* w, double* loads)
{
    int nb = o->nb;
    if (nb <= 0) return;
    if (c) memcpy(c, o->bc, 3 * nb * sizeof(double));
    if (q) memcpy(q, o->bq, 4 * nb * sizeof(double));
    if (v) memcpy(v, o->bv, 3 * nb * sizeof(double));
    if (w) memcpy(w, o->bw, 3 * nb * sizeof(double));
    if (loads) memcpy(loads, o->bloads, 6 * nb * sizeof(double));
}
void orc_get_grid(const orc* o, uint64_t* keys, int* ids)
{
    if (keys) memcpy(keys, o->skey, o->nc * sizeof(uint64_t));
    if (ids) memcpy(ids, o->sid, o->nc * sizeof(int));
}
void orc_get_triangle_grid(const orc* o, uint64_t* keys, int* ids)
{
    if (keys) memcpy(keys, o->tkey, o->tentries * sizeof(uint64_t));
    if (ids) memcpy(ids, o->tid, o->tentries * sizeof(int));
}
void orc_get_world_triangles(const orc* o, double* tw, double* aabb)
{
    if (tw) memcpy(tw, o->tw, 15 * (size_t)o->nt * sizeof(double));
    if (aabb) memcpy(aabb, o->taabb, 6 * (size_t)o->nt * sizeof(double));
}
void orc_get_components(const orc* o, double* pos, double* vel, double* vh, double* off)
{
    if (pos) memcpy(pos, o->cpos, 3 * o->nc * sizeof(double));
    if (vel) memcpy(vel, o->cvel, 3 * o->nc * sizeof(double));
    if (vh) memcpy(vh, o->cvh, 3 * o->nc * sizeof(double));
    if (off) memcpy(off, o->coff, 3 * o->nc * sizeof(double));
}
/* Same state as the reference after gpuUpdateComponents (for the
 * component-transform known answers, tests/component_transform_test.cu). */
void orc_update_components(orc* o) { update_components(o); }
void orc_set_half(orc* o, const double* vh, const double* wh)
{
    if (vh) memcpy(o->vh, vh, 3 * o->n * sizeof(double));
    if (wh) memcpy(o->wh, wh, 3 * o->n * sizeof(double));
}
void orc_get_history(const orc* o, int kind, uint64_t* keys, int* last, double* val)
{
    const hist_t* h = kind == 0 ? &o->hp : (kind == 1 ? &o->hw : &o->hb);
    size_t s = (size_t)o->nc * h->slots;
    if (keys) memcpy(keys, h->keys, s * sizeof(uint64_t));
    if (last) memcpy(last, h->last, s * sizeof(int));
    if (val) memcpy(val, h->val, s * 9 * sizeof(double));
}
void orc_get_stats(const orc* o, dem_step_stats* s) { *s = o->stats; }
void orc_get_regime_state(const orc* o, int* st) { if (o->nb > 0) memcpy(st, o->regime_state, (size_t)o->nb * o->nc * sizeof(int)); }
double orc_mesh_size(const orc* o) { return o->mesh; }
int orc_step_index(const orc* o) { return o->step_index; }
