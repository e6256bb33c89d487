// dem_kernels.cuh -- device data layout and kernel launchers of the engine.
//
// HBM layout (one engine, all scenes concatenated):
//   owners      input-order SoA, FP64 (positions, velocities, quaternions,
//               half-step state, accelerations, constants)
//   components  input-order SoA; for plain spheres the position and velocity
//               pointers alias the owner arrays (no copy kernel runs)
//   cell table  dense int32 start table over the per-step cell box of every
//               scene (segmented: scene s owns [offset_s, offset_s + cells_s))
//   records     per sorted position t (cell order), packed double4/float4
//               rows of the component the contact kernels read
//   history     reference slot layout [component][slot] (keys u64, last-seen
//               i32, 9 values of T per slot) updated in place
//   contacts    flat list of (i sorted pos, j sorted pos, history slot) with
//               per-contact force/torque rows of T
#pragma once

#include "dem_device.cuh"

#include <cstdint>
#include <cuda_runtime.h>

namespace demgb {

// Error word bits (reported at diagnostic points).
enum : unsigned {
    kErrKeyRange = 1u,        // cell coordinate outside the signed 21-bit range
    kErrCellCapacity = 2u,    // dense cell table too small for the cell box
    kErrTriCapacity = 4u,     // triangle grid entries beyond capacity
    kErrTriRange = 8u,        // triangle cell range overflow (reference :422-450)
    kErrScanWait = 16u,       // a single-pass scan gave up waiting for a predecessor tile
};

// Single-pass scan state (decoupled look-back).  Tiles are claimed in order
// through ctl[0]; each publishes a status word (value << 32 | epoch << 2 |
// flag: 1 aggregate, 2 inclusive prefix); ctl[1] counts finished blocks and
// the last one resets ctl[0..1] and advances the epoch ctl[2], so the words
// of an earlier launch read as not ready.  One state per concurrent scan.
struct ScanState {
    unsigned long long* status;  // [max_tiles]
    unsigned* ctl;               // [3]: ticket, blocks done, epoch
    int max_tiles;
};

// Sorted positions per tile of the particle-triangle item scan: 1,024 up to
// kPtWideTileComps components (fewer tiles to chain), 256 above (more
// resident blocks); the scan state is sized for the smaller tile.  On the
// 2M drum the wide tiles measured 1.047 -> 1.038 ms once the sweep, the
// particle law and the owner sum kept more blocks resident (0.3% slower
// before).
constexpr int kPtItemTile = 256;
constexpr int kPtItemTileWide = 1024;
constexpr int kPtWideTileComps = 4000000;

#ifdef __CUDACC__
constexpr int kScanSpinLimit = 1 << 20;

__device__ __forceinline__ unsigned long long scan_word(int value, unsigned epoch, unsigned flag)
{
    return ((unsigned long long)(unsigned)value << 32) | ((unsigned long long)(epoch & 0x3fffffffu) << 2) | flag;
}
__device__ __forceinline__ void scan_publish(const ScanState& st, int tile, int value, unsigned epoch, unsigned flag)
{
    atomicExch(st.status + tile, scan_word(value, epoch, flag));
}
// Exclusive prefix of `tile` (warp 0 of the block, all lanes get it): reads
// 32 predecessor words at a time, back to the nearest inclusive one.  Every
// wait is bounded; at the bound it sets kErrScanWait and returns what it has.
__device__ __forceinline__ int scan_lookback(const ScanState& st, int tile, unsigned epoch, unsigned* err)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int prefix = 0, top = tile - 1, spins = 0;
    while (true) {
        const int idx = top - lane;
        unsigned flag = 2u;  // before tile 0: an inclusive zero
        int val = 0;
        if (idx >= 0) {
            const unsigned long long w = atomicAdd(st.status + idx, 0ull);
            const bool current = ((w >> 2) & 0x3fffffffu) == (epoch & 0x3fffffffu);
            flag = current ? (unsigned)(w & 3u) : 0u;
            val = (int)(unsigned)(w >> 32);
        }
        const unsigned incl = __ballot_sync(FULL, flag == 2u);
        const unsigned waiting = __ballot_sync(FULL, flag == 0u);
        const int stop = incl ? __ffs(incl) - 1 : 31;
        const unsigned need = stop == 31 ? FULL : ((1u << (stop + 1)) - 1u);
        if (waiting & need) {
            if (++spins > kScanSpinLimit) {
                if (lane == 0) atomicOr(err, kErrScanWait);
                return prefix;
            }
            __nanosleep(32);
            continue;
        }
        int v = lane <= stop ? val : 0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
        prefix += v;
        if (incl) return prefix;
        top -= 32;
    }
}
#endif

struct Owners {
    int n;
    double *px, *py, *pz, *vx, *vy, *vz, *wx, *wy, *wz, *qw, *qx, *qy, *qz;
    double *ax, *ay, *az, *awx, *awy, *awz;
    double *vhx, *vhy, *vhz, *whx, *why, *whz, *hqw, *hqx, *hqy, *hqz;
    double *mass, *ix, *iy, *iz, *radius;
    double *inv_mass, *inv_ix, *inv_iy, *inv_iz;
    double* mg;  // [n][3] field force m*g of the owner's scene (0 without gravity)
    unsigned char* iso;  // isotropic inertia (Ix == Iy == Iz): no gyroscopic terms
    float* inv_i_f;      // FP32 inverse inertia of isotropic owners (mixed form)
    int *id, *status, *scene;
    double *ugx, *ugy, *ugz;  // universal-gravitation field force (optional)
};

struct Comps {
    int n;
    int sphere;  // 1: component c is owner c with zero offset
    int *owner, *cid, *ostart;
    double *radius, *bx, *by, *bz;                                      // body-frame offset
    double *x, *y, *z, *vx, *vy, *vz, *vhx, *vhy, *vhz, *ox, *oy, *oz;  // world (aliases for spheres)
};

// Per-scene constants.
struct SceneC {
    MatC pp, pt, pw;
    MatF ppf, ptf, pwf;
    double g[3];
    // Cell edge (cell factor x the scene's largest component radius), its
    // inverse and the triangle-grid padding (the largest radius): each scene
    // of a batch is gridded exactly as it would be alone.
    double mesh, inv_mesh, pad;
    float mesh_f, margin_f, inv_mesh_f;
    // Neighbour lists: the skin (FP32, m) and (skin / 2)^2 (FP64, m^2), the
    // displacement since the lists' build that calls for a rebuild.  The
    // skin keeps r_i + r_j + skin within the cell edge, so the build sweep's
    // 27 cells hold every pair it must list.
    float skin_f;
    double nl_half2;
    int grav;
    int wall_begin, wall_count;
    int body_begin, body_count;
};

struct Grid {
    const SceneC* sc;  // per-scene cell edge
    int capacity;      // cells in the dense table
    int nscenes;
    uint64_t* ckey;
    int *clin, *crank;
    int *cell_count, *cell_start;
    int *sorted_id, *pos_of, *sorted_tmp;
    uint64_t* sorted_key;
    int* scene_box;     // [S][6]
    int* scene_layout;  // [S][8]: min xyz, n xyz, offset, cells
    int* total_cells;   // [1]
    int* nvalid;        // [1] = cell_start[total_cells]
    unsigned* err;
    ScanState scan;    // the cell start table's single-pass scan
};

// 32-byte aligned row of four doubles (one full sector per row).
struct __align__(32) D4 {
    double x, y, z, w;
};

// Velocity rows are D4 in the FP64 form and float4 in the mixed form (the
// law reads them as FP32 there; the particle-triangle law reads FP64 state
// from the owner and component arrays instead).
struct Recs {
    D4 *pos, *v, *vm, *w, *wm, *off;  // off: clumps only
    float4 *vf, *vmf, *wf, *wmf;      // mixed form
    int4* meta;                             // c, owner, component id, scene
    int4* cell;                             // cx, cy, cz, lin
    float4* relf;                           // position relative to the cell origin, radius
};

// History values: 9 per slot (roll, tangent, twist vectors), stored with a
// stride of 12 so a slot starts on a 16-byte boundary and moves as three
// float4 (FP32) or five double2 (FP64) accesses.
constexpr int kHV = 12;
constexpr int kNL = 32;  // neighbour-list capacity per component

// One history kind.  Keys and last-seen steps are slot-major, slot s of
// component c at s * nc + c, so a warp of neighbouring components reads one
// slot in a few lines; the values are component-major, slot s of component
// c at (c * slots + s) * kHV, so one contact side reads its 9 values from one
// row.  The "slot index" that contact lists and tapes carry is c * slots + s.
template <typename T> struct Hist {
    uint64_t* key;
    int* last;
    T* val;
    int* hw;  // per component: 1 + highest occupied slot
    int nc;   // components (the key and last-seen stride)
};
template <typename T> __host__ __device__ inline size_t hslot(const Hist<T>& h, int c, int s)
{
    return (size_t)s * h.nc + c;
}

struct Walls {
    int count;      // walls of all scenes
    double *o, *n;  // [nw][3]
    float4* plane;  // [nw] FP32 (normal, normal . origin) for the prefilter
};

struct Tris {
    int nt;
    int* body;
    double* local;  // [t][15]
    double* world;  // [t][16] v1..v4, normal, pad
    int* trange;    // [t][6] padded-AABB cell range (lo xyz, hi xyz); lo.x = INT_MAX outside the key range
    float4* tf;     // [t][2] FP32 copies for prefilters: (normal, normal . v2), (centroid of v2..v4, circumradius)
    int* scene;     // per triangle
    int capacity;   // triangle grid entry capacity
    int *tcell_count, *tcell_cursor, *tcell_start, *ttri, *ttri_tmp, *tlin_tmp;
    ScanState scan;  // the triangle start table's single-pass scan (its own: it builds beside the particle grid)
};

struct Bodies {
    int nb;
    double *c, *q, *v, *w;  // [nb][3/4/3/3] device copies uploaded per step
    int* scene;
};

struct Counters {
    int* pcontacts;     // per step
    int* pover;         // cumulative
    int* bover;         // cumulative (wall + body, as the reference)
    int* phigh;         // per step
    int* bhigh;         // per step
    int* tgover;        // per build
    int* ct_total;      // contacts this step
    int* pt_ctotal;     // PT components touching a triangle this step
    int* wl_total;      // components with a candidate wall this step
    int* step;          // contact step index
    int pt_warp_items;  // PT: warp-per-item kernel up to this many contact items
    int sweep_bps;      // sweep blocks per SM (grid-stride), 0 = one thread per component
    int gather_bps;     // gather blocks of 256 per SM (grid-stride)
    // Neighbour lists (nl_on): per component up to kNL partner components
    // within r_i + r_j + skin at the last build, and the build positions.
    // nl_flag[0] nonzero: this step sweeps the cells and rebuilds the lists
    // (set by the host, by a displacement past skin/2, or by an overflow);
    // nl_flag[1]: the last build overflowed a list.
    int nl_on;
    int* nl_flag;       // [0] rebuild this step, [1] overflow at the last build, [2] builds so far, [3] movers this step
    int* nl_hot;        // per cell of the dense table: the step at which it held a mover
    int nl_limit;       // movers beyond which every list is rebuilt
    int* nl_cnt;
    int* nl_idx;
    double* nl_xref;
    int pp_bps;         // particle-law blocks of 256 per SM (grid-stride), 0 = 16
};

// Reverse sweep (dem_adjoint.cu).  Owner state S of one step, [field][owner]:
// x 3, q 4, v 3, w (body frame) 3, vh 3, wh 3, hq 4, a 3, aw 3.
constexpr int kAdjX = 0, kAdjQ = 3, kAdjV = 7, kAdjW = 10, kAdjVH = 13, kAdjWH = 16, kAdjHQ = 19, kAdjA = 23,
              kAdjAW = 26, kAdjFields = 29;
// post-advance state the laws see: x1, q1, v1, w1 (body frame), midpoint v
// and w (body frame), and the world-frame spins R(q1) w1 and R(q1) w_mid
constexpr int kPX = 0, kPQ = 3, kPV = 7, kPW = 10, kPMV = 13, kPMW = 16, kPEW = 19, kPEMW = 22, kPFields = 25;
// adjoints of the post-advance state, of the midpoint velocities, of the
// total force and world torque of each owner, and of its two world-frame
// spins (the contact kernels add these; the owner step turns them into
// quaternion and spin adjoints)
constexpr int kTX = 0, kTQ = 3, kTV = 7, kTW = 10, kTMV = 13, kTMW = 16, kTF = 19, kTTau = 22, kTEW = 25, kTEMW = 28,
              kTFields = 31;
// material adjoints per contact class: kN, mu, log epsN, log epsS, muT, muR
constexpr int kAdjParams = 6;

// Adjoint tape of one step (FP64 form, written only while the engine tapes a
// recomputed step): per particle contact side (component, partner component,
// history slot index, 1 if the slot was acquired this step) and the slot's
// history before the law; the same for wall contacts (component, wall,
// slot index, new).  With `slot` set, the arrays hold every step of a
// segment and the step is the device value *slot (tape_at applies it), so
// one captured graph serves all steps.
struct StepTape {
    unsigned char* pp_new;  // per contact list entry, written by the sweep
    int4* pp;
    double* pp_h;           // [entry][kHV]
    int pp_cap;
    int4* pw;
    double* pw_h;
    int pw_cap;
    int* pw_count;
    int* overflow;
    int* pp_count;          // particle entries of the step (read by the reverse kernels)
    const int* slot;        // device step index, or null: the pointers are the step's own
    int4* pb;               // particle-body manifolds: component, body, history index (c * kBSlots + slot), new
    int* pb_tri;            // [entry][kPbTri]: triangle count, then the triangles (those with an area share)
    double* pb_h;           // [entry][kHV] history before the step
    int pb_cap;
    int* pb_count;
};
constexpr int kPbTri = kPbTris + 1;

#ifdef __CUDACC__
__device__ __forceinline__ StepTape tape_at(StepTape t)
{
    if (t.slot) {
        const size_t k = (size_t)*t.slot;
        t.pp += k * t.pp_cap;
        t.pp_h += k * t.pp_cap * kHV;
        t.pw += k * t.pw_cap;
        t.pw_h += k * t.pw_cap * kHV;
        t.pw_count += k;
        if (t.pp_count) t.pp_count += k;
        if (t.pb) {
            t.pb += k * t.pb_cap;
            t.pb_tri += k * t.pb_cap * kPbTri;
            t.pb_h += k * t.pb_cap * kHV;
            t.pb_count += k;
        }
        t.slot = nullptr;
    }
    return t;
}
#endif

template <typename T> struct Contacts {
    int4* ent;      // ti, tj, slot, -
    T* res;         // [k][6]
    int *off, *cnt; // per component
    int capacity;
    double* wres;   // [c][6] wall force/torque per component (valid where wflag)
    unsigned char* wflag;  // per component: nonzero wall force/torque this step
    int2* wlist;           // components with a candidate wall: (component, wall mask)
    int* pt_index;  // per component: contact item or -1
    int* pt_clist;      // contact item k -> sorted position
    int* pt_ctotal_ptr; // [1] contact items this step
    ScanState pt_scan;  // single-pass scan of the contact-item compaction
    double* pt_res; // [component][6] particle-side PT load (valid where pt_index >= 0)
    double* pt_body;    // [contact item][nbs][kPtRecord]
    double* pt_out;     // [contact item][nbs][25] optional output detail
    int nbs;            // max bodies per scene
    StepTape tape;      // adjoint tape (all null when not taping)
};

struct BodyOut {
    double* partial;   // [nb][G][kPtRecord]
    double* result;    // [nb][kPtRecord]: load 6, count, maxdepth, fz, regime 7, micro 22 (see kernels)
    unsigned long long* reg_int;  // [nb][7]
    double* micro_int;            // [nb][22]
    unsigned long long* native_steps;
    int groups;
};

// ------------------------------------------------------------- launchers
void launch_update_components(const Comps& c, const Owners& o, cudaStream_t s);
// The particle grid in two parts: cell keys and the per-scene cell layout
// (all the triangle grid needs), then the counting sort.
void launch_grid_layout(const Comps& c, const Owners& o, const Grid& g, cudaStream_t s);
void launch_grid_sort(const Comps& c, const Owners& o, const Grid& g, int sm_count, cudaStream_t s);
void launch_scan(const int* in, int* out, const int* n_dev, int* tile_sums, int sm_count, cudaStream_t s);
// Single-pass exclusive scan of in[0, n) into out[0, n] (out[n] = total).
// Failure detection of the single-pass scans without a fault: one warp looks
// back from tile 1 at a tile 0 that never publishes; the bounded wait gives
// up and sets kErrScanWait in *err.  `status` holds one zero word.
void launch_scan_wait_probe(unsigned long long* status, unsigned* err, cudaStream_t s);
void launch_scan1(const int* in, int* out, const int* n_dev, const ScanState& st, unsigned* err, int sm_count,
                  cudaStream_t s);
void launch_tri_transform(const Tris& t, const Bodies& b, const SceneC* sc, cudaStream_t s);
void launch_tri_build(const Tris& t, const Bodies& b, const Grid& g, int* tgover, int sm_count, cudaStream_t s);
void launch_universal_gravity(const Owners& o, cudaStream_t s);
void launch_leapfrog_init(const Owners& o, double half_dt, cudaStream_t s);
void launch_advance(const Owners& o, double dt, cudaStream_t s);
void launch_finish(const Owners& o, double dt, cudaStream_t s);
// launch_finish in two parts: the half-step velocities, then the half-step
// quaternion rate (which launch_advance_rest also computes, from the same
// values, before it advances the quaternion).
void launch_finish_vel(const Owners& o, double dt, cudaStream_t s);
void launch_finish_rot(const Owners& o, double dt, cudaStream_t s);
// finishParticleStep of one step fused with advanceParticles of the next.
// launch_finish followed by launch_advance, in two parts: positions (what
// the next particle grid needs), then the rest of the advance.
void launch_finish_advance_pos(const Owners& o, double dt, cudaStream_t s);
void launch_advance_rest(const Owners& o, double dt, int sm_count, cudaStream_t s);
// launch_advance in two parts: positions, then quaternions and velocities.
void launch_advance_pos(const Owners& o, double dt, cudaStream_t s);
void launch_advance_rot(const Owners& o, double dt, int sm_count, cudaStream_t s);
// reset != 0: clear the per-step counters; 0: advance the contact step index.
void launch_step_counter(const Counters& k, int reset, cudaStream_t s);

// Owner-state snapshots [29][n]; with `slot`, into S + *slot * 29 n.
void launch_adj_snapshot(const Owners& o, double* S, cudaStream_t s, const int* slot = nullptr);
void launch_adj_restore(const Owners& o, const double* S, cudaStream_t s);
// Compact checkpoint of one history kind: the occupied prefix [0, hw[c]) of
// every component c at offset off[c] (an exclusive scan of hw), and back
// (slots between the stored and the live mark are cleared).
void launch_ckpt_pack(const Hist<double>& h, int slots, int nc, const int* off, uint64_t* key, int* last, double* val,
                      int sm_count, cudaStream_t s);
void launch_ckpt_unpack(const Hist<double>& h, int slots, int nc, const int* hw, const int* off, const uint64_t* key,
                        const int* last, const double* val, int sm_count, cudaStream_t s);
// The rigid bodies of the reverse mode: the forward run's body records
// ([step][body][39]: the pose the evaluation used, the loads, the state after
// the half update), constants ([body][5]: mass, principal inertia, state),
// the adjoints ([body][35]) and the triangles' body-frame records.  The
// global step of a tape slot is *base + slot (base null: slot 0 is step 0).
struct AdjBodies {
    int nb;
    const double* rec;
    const double* cst;
    double* L;
    const int* base;
    const double* local;
    double dt;
};
// One reverse step.  npp / npw / npb < 0: the counts are the tape's own
// (at the device slot) and S, S1 are taken at *tp.slot and *tp.slot + 1 of
// the snapshot array S.  `grads` holds [nscenes][3][kAdjParams] material
// gradients (particle, wall, triangle).  With rigid bodies, s2 and three
// events make the step a DAG (the bodies' reverse beside the owners').
void launch_adj_step(const Comps& c, const Owners& o, const SceneC* sc, const Walls& w, const StepTape& tp, int npp,
                     int npw, int npb, const double* S, const double* S1, const double* L, double* Lp, double* P,
                     double* T, double* lh_pp, double* lh_pw, double* lh_pb, const AdjBodies& ab, double dt,
                     double dt_eff, int init, double* grads, int nscenes, int sm_count, cudaStream_t s,
                     cudaStream_t s2 = nullptr, cudaEvent_t* ev = nullptr, bool fp32 = false);
// Recompute: the body pose of the tape's step (record *base + *slot; null
// pointers: record 0) into the engine's body arrays.
void launch_adj_body_pose(const Bodies& b, const double* rec, const int* base, const int* slot, cudaStream_t s);
void launch_set_int(int* p, int v, cudaStream_t s);
// Device step index of a taped segment: add `delta`.
void launch_adj_slot_add(int* slot, int delta, cudaStream_t s);
// Before a taped step: zero its wall entry count.  After it: record its
// particle entry count (the contact total) and move to the next step.
void launch_adj_tape_begin(int* pw_count, int* pb_count, const int* slot, cudaStream_t s);
void launch_adj_tape_end(int* pp_count, const int* ct_total, int* slot, cudaStream_t s);

// The sorted records: geometry (positions only; all the sweep reads), then
// velocities (after the rotational advance).
// bps: blocks of 256 per SM (grid-stride), so the kernels beside them keep slots.
void launch_gather_geom(const Comps& c, const Owners& o, const Grid& g, const Recs& r, int sm_count, int bps,
                        const Counters& k, cudaStream_t s);
template <typename T>
void launch_gather_vel(const Comps& c, const Owners& o, const Grid& g, const Recs& r, double dt_eff, int sm_count,
                       int bps, cudaStream_t s);
// T: particle-particle and wall law / history type; TB: particle-triangle
// law, area and body history type.  `stage` selects kernels (1 expiry and
// walls, 2 sweep, 4 particle law, 8 particle-triangle items, 16
// particle-triangle law) so callers can time them separately; 31 runs all
// in order.
template <typename T, typename TB>
void launch_contacts(const Comps& c, const Owners& o, const Grid& g, const Recs& r, const SceneC* sc, const Walls& w,
                     const Tris& t, const Bodies& b, Hist<T> hp, Hist<T> hw, Hist<TB> hb, Contacts<T> ct,
                     const Counters& k, double dt_eff, int block, int sm_count, cudaStream_t s, int stage = 31);
template <typename T>
void launch_owner_sum(const Comps& c, const Owners& o, const SceneC* sc, Contacts<T> ct, bool outputs, double* fc,
                      double* ff, double* fw, double* ft, cudaStream_t s);
template <typename T>
void launch_body_reduce(const Recs& r, const SceneC* sc, const Bodies& b, Contacts<T> ct, BodyOut bo, bool interval,
                        cudaStream_t s);
template <typename T>
void launch_body_outputs(const Comps& c, const Owners& o, const Bodies& b, const SceneC* sc, Contacts<T> ct,
                         double* bp, double* bd, cudaStream_t s);

constexpr int kBodyFieldCount = 38;  // body reduction record, see dem_contact.cu

}  // namespace demgb
