// dem_grid.cu -- cell hash, counting sort with cell start tables, triangle
// grid, leapfrog and quaternion integration.
//
// The particle grid replaces the reference's thrust::sequence +
// thrust::sort_by_key over 63-bit packed cell keys followed by per-lookup
// binary searches (src/cuda/cuda_grid_backend.cu:121-145,
// src/cuda/cuda_contact_backend.cu:144-176,1131-1135).  Each step:
//   1. cell key of every component (same floor(x * 1/mesh), same range check)
//      and the per-scene cell box (warp-reduced atomics);
//   2. a dense per-scene cell layout over that box (one block);
//   3. counting sort: per-cell atomic count + rank, device-wide exclusive
//      scan (the start table), scatter;
//   4. per cell, its entries are put in ascending component order.
// Step 4 makes the result equal to a stable sort of the keys over component
// indices, i.e. the reference's sortedCellKey / sortedEntityId, and the scan
// is the cell start/end table the contact kernels index directly.
#include "../../include/dem_gb300.h"
#include "dem_kernels.cuh"

#include <algorithm>
#include <climits>

namespace demgb {

namespace {

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanBlock * kScanItems;

__device__ __forceinline__ int warp_min(int v)
{
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max(int v)
{
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide exclusive scan of one int per thread (blockDim multiple of 32).
__device__ int block_exclusive_scan(int v, int& total)
{
    __shared__ int warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < nw ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    total = warp_sums[nw - 1];
    const int base = wid > 0 ? warp_sums[wid - 1] : 0;
    __syncthreads();
    return base + x - v;
}

// ------------------------------------------------------------------ keys
// updateComponentsKernel (src/cuda/cuda_particle_backend.cu:116-147).
__global__ void k_update_components(Comps c, Owners o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int w = c.owner[i];
    const double qw = o.qw[w], qx = o.qx[w], qy = o.qy[w], qz = o.qz[w];
    const V3<double> off = rot_iv(qw, qx, qy, qz, mk(c.bx[i], c.by[i], c.bz[i]));
    c.ox[i] = off.x; c.oy[i] = off.y; c.oz[i] = off.z;
    c.x[i] = o.px[w] + off.x; c.y[i] = o.py[w] + off.y; c.z[i] = o.pz[w] + off.z;
    const V3<double> ow = rot_iv(qw, qx, qy, qz, mk(o.wx[w], o.wy[w], o.wz[w]));
    c.vx[i] = o.vx[w] + ow.y * off.z - ow.z * off.y;
    c.vy[i] = o.vy[w] + ow.z * off.x - ow.x * off.z;
    c.vz[i] = o.vz[w] + ow.x * off.y - ow.y * off.x;
    const V3<double> hw = rot_iv(qw, qx, qy, qz, mk(o.whx[w], o.why[w], o.whz[w]));
    c.vhx[i] = o.vhx[w] + hw.y * off.z - hw.z * off.y;
    c.vhy[i] = o.vhy[w] + hw.z * off.x - hw.x * off.z;
    c.vhz[i] = o.vhz[w] + hw.x * off.y - hw.y * off.x;
}

// The reference's cell coordinates, floor(x * inv_mesh) in FP64 per axis,
// all finite and inside [-2^20, 2^20 - 1].  Out of line, so its FP64 work is
// issued only by warps with a component that the FP32 estimate leaves open.
__device__ __noinline__ bool cell_coords_exact(double x, double y, double z, double inv_mesh, int& cx, int& cy,
                                               int& cz)
{
    const double minCell = -(double)(1 << 20), maxCell = (double)((1 << 20) - 1);
    const double fx = floor(x * inv_mesh), fy = floor(y * inv_mesh), fz = floor(z * inv_mesh);
    const bool ok = isfinite(fx) && isfinite(fy) && isfinite(fz) && fx >= minCell && fx <= maxCell &&
                    fy >= minCell && fy <= maxCell && fz >= minCell && fz <= maxCell;
    if (ok) { cx = (int)fx; cy = (int)fy; cz = (int)fz; }
    return ok;
}

// FP32 estimate of floor(x * inv_mesh).  q = fl32(fl32(x) * fl32(inv_mesh))
// is within 1.8e-7 |q| of the FP64 product (three FP32 roundings and one
// FP64 one), so when q - e and q + e (e = 4e-7 |q|, which also covers the
// rounding of q -+ e) have the same floor, that floor is the FP64 one.
// False when open: near a cell face, at 0, or not well inside the key range
// (|q| < 1e6 < 2^20), non-finite included.
// floor(q) for |q| < 2^22 with FP32 adds only: adding and removing 1.5 * 2^23
// rounds q to the nearest integer, which is one too high when above q.
__device__ __forceinline__ float floor_small(float q)
{
    const float r = __fadd_rn(__fadd_rn(q, 12582912.0f), -12582912.0f);
    return r > q ? r - 1.0f : r;
}
__device__ __forceinline__ bool cell_coord_f32(double x, float inv_mesh_f, int& c)
{
    const float q = f32_rn(x) * inv_mesh_f;
    const float e = fmaf(4.0e-7f, fabsf(q), 1.0e-30f);
    const float lo = floor_small(q - e), hi = floor_small(q + e);
    // the integer of lo (|lo| < 2^22) in the low mantissa bits of lo + 1.5 * 2^23
    c = __float_as_int(__fadd_rn(lo, 12582912.0f)) - 0x4B400000;
    return fabsf(q) < 1.0e6f && lo == hi;
}

// computeComponentKeysKernel (src/cuda/cuda_grid_backend.cu:51-71) plus the
// per-scene cell box.
// Grids of k_cell_keys above this many blocks read the cell box before
// updating it.
constexpr unsigned kBoxCheckBlocks = 2048;

__global__ void k_cell_keys(Comps c, Owners o, Grid g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = false;
    int cx = 0, cy = 0, cz = 0, s = INT_MAX;
    if (i < c.n) {
        const int sc = o.scene[c.owner[i]];
        const SceneC& S = g.sc[sc];
        const double x = c.x[i], y = c.y[i], z = c.z[i];
        ok = cell_coord_f32(x, S.inv_mesh_f, cx) & cell_coord_f32(y, S.inv_mesh_f, cy) &
             cell_coord_f32(z, S.inv_mesh_f, cz);
        if (!ok) ok = cell_coords_exact(x, y, z, S.inv_mesh, cx, cy, cz);
        if (ok) {
            s = sc;
            g.ckey[i] = pack_cell(cx, cy, cz);
            g.clin[i] = 0;
        } else {
            g.ckey[i] = 0;
            g.clin[i] = -1;
            atomicOr(g.err, kErrKeyRange);
        }
    }
    // Cell box: warp min/max, then one set of atomics per scene and block.
    __shared__ int sh_box[8][7];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int smin = warp_min(ok ? s : INT_MAX);
    const bool uniform = __all_sync(0xffffffffu, !ok || s == smin);
    if (uniform) {
        const int a0 = warp_min(ok ? cx : INT_MAX), a1 = warp_min(ok ? cy : INT_MAX), a2 = warp_min(ok ? cz : INT_MAX);
        const int b0 = warp_max(ok ? cx : INT_MIN), b1 = warp_max(ok ? cy : INT_MIN), b2 = warp_max(ok ? cz : INT_MIN);
        if (lane == 0) {
            sh_box[wid][0] = smin; sh_box[wid][1] = a0; sh_box[wid][2] = a1; sh_box[wid][3] = a2;
            sh_box[wid][4] = b0; sh_box[wid][5] = b1; sh_box[wid][6] = b2;
        }
    } else {
        if (lane == 0) sh_box[wid][0] = INT_MAX;
        if (ok) {
            int* box = g.scene_box + 6 * s;
            atomicMin(box + 0, cx); atomicMin(box + 1, cy); atomicMin(box + 2, cz);
            atomicMax(box + 3, cx); atomicMax(box + 4, cy); atomicMax(box + 5, cz);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) {
            const int sc = sh_box[w][0];
            if (sc == INT_MAX) continue;
            int a[3] = {sh_box[w][1], sh_box[w][2], sh_box[w][3]}, b[3] = {sh_box[w][4], sh_box[w][5], sh_box[w][6]};
            for (int v = w + 1; v < nw; ++v) {
                if (sh_box[v][0] != sc) continue;
                for (int k = 0; k < 3; ++k) { a[k] = min(a[k], sh_box[v][1 + k]); b[k] = max(b[k], sh_box[v][4 + k]); }
                sh_box[v][0] = INT_MAX;
            }
            // The box only moves towards the block's values.  On large grids
            // an atomic that the current value already satisfies is skipped
            // (most blocks of a scene change none of the six, and thousands
            // of atomics on six words serialise); the six loads go out
            // together, past L1, and a stale value only costs an atomic.
            // Small grids issue the atomics at once (the loads would only
            // add their latency to the block's end).
            int* box = g.scene_box + 6 * sc;
            int cur[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
            if (gridDim.x > kBoxCheckBlocks) {
#pragma unroll
                for (int k = 0; k < 6; ++k) cur[k] = __ldcg(box + k);
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (a[k] < cur[k]) atomicMin(box + k, a[k]);
                if (b[k] > cur[3 + k]) atomicMax(box + 3 + k, b[k]);
            }
        }
    }
}

// Dense segmented cell layout: scene s owns cells [offset, offset + cells).
__global__ void k_layout(Grid g)
{
    if (threadIdx.x == 0) {
        long long off = 0;
        for (int s = 0; s < g.nscenes; ++s) {
            const int* box = g.scene_box + 6 * s;
            int* lay = g.scene_layout + 8 * s;
            long long cells = 0;
            long long nx = 0, ny = 0, nz = 0;
            if (box[0] <= box[3]) {
                nx = (long long)box[3] - box[0] + 1;
                ny = (long long)box[4] - box[1] + 1;
                nz = (long long)box[5] - box[2] + 1;
                // each extent is at most 2^21, so nx * ny * nz can reach 2^63
                // and wrap; the product is only formed once nx * ny fits
                if (nx * ny > (long long)g.capacity || off + nx * ny * nz > (long long)g.capacity)
                    atomicOr(g.err, kErrCellCapacity);
                else
                    cells = nx * ny * nz;
            }
            lay[0] = box[0]; lay[1] = box[1]; lay[2] = box[2];
            lay[3] = cells ? (int)nx : 0; lay[4] = cells ? (int)ny : 0; lay[5] = cells ? (int)nz : 0;
            lay[6] = (int)off; lay[7] = (int)cells;
            off += cells;
        }
        *g.total_cells = (int)off;
    }
    __syncthreads();
    for (int s = threadIdx.x; s < g.nscenes; s += blockDim.x) {
        int* box = g.scene_box + 6 * s;
        box[0] = box[1] = box[2] = INT_MAX;
        box[3] = box[4] = box[5] = INT_MIN;
    }
}

__device__ __forceinline__ int cell_lin(const int* lay, int cx, int cy, int cz)
{
    return lay[6] + ((cx - lay[0]) * lay[4] + (cy - lay[1])) * lay[5] + (cz - lay[2]);
}

__global__ void k_cell_count(Comps c, Owners o, Grid g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n || g.clin[i] < 0) return;
    const int s = o.scene[c.owner[i]];
    const int* lay = g.scene_layout + 8 * s;
    if (lay[7] == 0) { g.clin[i] = -1; return; }
    int cx, cy, cz;
    unpack_cell(g.ckey[i], cx, cy, cz);
    const int lin = cell_lin(lay, cx, cy, cz);
    g.clin[i] = lin;
    g.crank[i] = atomicAdd(g.cell_count + lin, 1);
}

__global__ void k_scatter(Comps c, Grid g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int lin = g.clin[i];
    if (lin < 0) return;
    g.sorted_tmp[g.cell_start[lin] + g.crank[i]] = i;
}

// Final position of a component inside its cell = number of cell members
// with a smaller index, so every cell lists its members in ascending
// component order: the result equals a stable sort of the cell keys.  Also
// writes the inverse permutation and sorted keys, and restores the zero
// count invariant of the cell table.
__global__ void k_place(Comps c, Grid g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *g.nvalid = g.cell_start[*g.total_cells];
    if (i >= c.n) return;
    const int lin = g.clin[i];
    if (lin < 0) return;
    const int b = g.cell_start[lin], e = g.cell_start[lin + 1];
    int rank = 0;
    for (int p = b; p < e; ++p) rank += g.sorted_tmp[p] < i;
    const int pos = b + rank;
    g.sorted_id[pos] = i;
    g.pos_of[i] = pos;
    g.sorted_key[pos] = g.ckey[i];
    g.cell_count[lin] = 0;
}

// ------------------------------------------------------------------ scan
__global__ void k_scan_reduce(const int* in, const int* n_dev, int* tile_sums)
{
    const int n = *n_dev;
    const int ntiles = (n + kScanTile - 1) / kScanTile;
    __shared__ int red[32];
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int base = tile * kScanTile + threadIdx.x * kScanItems;
        int s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) s += (base + k < n) ? in[base + k] : 0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            int v = red[threadIdx.x];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (threadIdx.x == 0) tile_sums[tile] = v;
        }
        __syncthreads();
    }
}

__global__ void k_scan_tile_sums(int* tile_sums, const int* n_dev)
{
    const int n = *n_dev;
    const int ntiles = (n + kScanTile - 1) / kScanTile;
    int running = 0;
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < ntiles ? tile_sums[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, total);
        if (i < ntiles) tile_sums[i] = running + ex;
        running += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sums[ntiles] = running;
}

__global__ void k_scan_apply(const int* in, int* out, const int* n_dev, const int* tile_sums)
{
    const int n = *n_dev;
    const int ntiles = (n + kScanTile - 1) / kScanTile;
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = tile_sums[ntiles];
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int base = tile * kScanTile + threadIdx.x * kScanItems;
        int v[kScanItems];
        int s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) { v[k] = (base + k < n) ? in[base + k] : 0; s += v[k]; }
        int total;
        int ex = block_exclusive_scan(s, total) + tile_sums[tile];
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (base + k < n) out[base + k] = ex;
            ex += v[k];
        }
        __syncthreads();
    }
}

// ------------------------------------------------------ single-pass scan
// One launch instead of reduce / tile sums / apply: persistent blocks claim
// 4096-int tiles in order, sum them, publish the aggregate, look back over
// the predecessors' status words (ScanState, scan_lookback) and write the
// tile's exclusive prefixes.
constexpr int kScan1Block = 512;
constexpr int kScan1Items = 8;
constexpr int kScan1Tile = kScan1Block * kScan1Items;

__global__ void __launch_bounds__(kScan1Block) k_scan1(const int* in, int* out, const int* n_dev, ScanState st,
                                                      unsigned* err)
{
    __shared__ int s_tile, s_prefix;
    const int n = *n_dev;
    const int ntiles = min((n + kScan1Tile - 1) / kScan1Tile, st.max_tiles);
    const unsigned epoch = st.ctl[2];
    if (n == 0 && blockIdx.x == 0 && threadIdx.x == 0) out[0] = 0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(st.ctl, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= ntiles) break;
        const int base = tile * kScan1Tile + threadIdx.x * kScan1Items;
        int v[kScan1Items];
        int sum = 0;
#pragma unroll
        for (int q = 0; q < kScan1Items; ++q) {
            v[q] = base + q < n ? in[base + q] : 0;
            sum += v[q];
        }
        int total;
        const int ex = block_exclusive_scan(sum, total);
        if (threadIdx.x == 0) scan_publish(st, tile, total, epoch, tile == 0 ? 2u : 1u);
        if (threadIdx.x < 32) {
            const int prefix = tile == 0 ? 0 : scan_lookback(st, tile, epoch, err);
            if (threadIdx.x == 0) {
                if (tile > 0) scan_publish(st, tile, prefix + total, epoch, 2u);
                s_prefix = prefix;
            }
        }
        __syncthreads();
        int run = s_prefix + ex;
#pragma unroll
        for (int q = 0; q < kScan1Items; ++q) {
            if (base + q < n) out[base + q] = run;
            run += v[q];
        }
        if (tile == ntiles - 1 && threadIdx.x == 0) out[n] = s_prefix + total;
        __syncthreads();  // s_tile, s_prefix are reused by the next tile
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(st.ctl + 1, 1u) == gridDim.x - 1) {
            st.ctl[0] = 0u;
            st.ctl[1] = 0u;
            atomicAdd(st.ctl + 2, 1u);
        }
    }
}

// ------------------------------------------------------------- triangles
// transformTrianglesKernel (src/cuda/cuda_body_backend.cu:71-112).
__global__ void k_tri_transform(Tris t, Bodies b, const SceneC* __restrict__ sc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t.nt) return;
    const int ib = t.body[i];
    const double* L = t.local + 15 * (size_t)i;
    double* W = t.world + 16 * (size_t)i;
    double g[3];
    tri_world(L, b.q[4 * ib], b.q[4 * ib + 1], b.q[4 * ib + 2], b.q[4 * ib + 3], b.c[3 * ib], b.c[3 * ib + 1],
              b.c[3 * ib + 2], W, g);
    if (t.tf) {
        const double na = W[12] * W[3] + W[13] * W[4] + W[14] * W[5];
        t.tf[2 * (size_t)i] = make_float4((float)W[12], (float)W[13], (float)W[14], (float)na);
        t.tf[2 * (size_t)i + 1] = make_float4((float)g[0], (float)g[1], (float)g[2], (float)W[15]);
    }
    // Padded-AABB cell range (countTriangleCellsKernel,
    // src/cuda/cuda_contact_backend.cu:409-452): floor((min - pad) / mesh)
    // .. floor((max + pad) / mesh) per axis, the same range check as a
    // particle key.  Computed once per triangle here; the grid kernels clip
    // it to the cell layout with integer arithmetic only.
    double mn[3] = {W[0], W[1], W[2]}, mx[3] = {W[0], W[1], W[2]};
    for (int k = 1; k < 4; ++k)
        for (int a = 0; a < 3; ++a) { mn[a] = fmin(mn[a], W[3 * k + a]); mx[a] = fmax(mx[a], W[3 * k + a]); }
    const SceneC& S = sc[t.scene[i]];
    const double minCell = -(double)(1 << 20), maxCell = (double)((1 << 20) - 1);
    int* R = t.trange + 6 * (size_t)i;
    bool ok = true;
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        const double l = floor((mn[a] - S.pad) * S.inv_mesh);
        const double h = floor((mx[a] + S.pad) * S.inv_mesh);
        if (!isfinite(l) || !isfinite(h) || l < minCell || h > maxCell) ok = false;
        lo[a] = ok ? (int)l : 0;
        hi[a] = ok ? (int)h : 0;
    }
    for (int a = 0; a < 3; ++a) { R[a] = lo[a]; R[3 + a] = hi[a]; }
    if (!ok) R[0] = INT_MAX;
}

// The stored cell range of triangle i clipped to the particle cell box of
// its scene: only those cells are ever looked up.
__device__ bool tri_cell_range(const Tris& t, const Grid& g, int i, int lo[3], int hi[3], const int*& lay)
{
    const int* R = t.trange + 6 * (size_t)i;
    lay = g.scene_layout + 8 * t.scene[i];
    if (lay[7] == 0) return false;
    for (int a = 0; a < 3; ++a) {
        lo[a] = max(R[a], lay[a]);
        hi[a] = min(R[3 + a], lay[a] + lay[3 + a] - 1);
        if (lo[a] > hi[a]) return false;
    }
    return true;
}

__device__ __forceinline__ bool tri_range_valid(const Tris& t, int i) { return t.trange[6 * (size_t)i] != INT_MAX; }

// One warp per triangle, the lanes over the cells of its padded AABB.
__global__ void k_tri_count(Tris t, Grid g, int* tgover)
{
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= t.nt) return;
    if (!tri_range_valid(t, i)) {
        if (lane == 0) {
            atomicAdd(tgover, 1);
            atomicOr(g.err, kErrTriRange);
        }
        return;
    }
    int lo[3], hi[3];
    const int* lay;
    if (!tri_cell_range(t, g, i, lo, hi, lay)) return;
    const int ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    const int cells = (hi[0] - lo[0] + 1) * ny * nz;
    for (int k = lane; k < cells; k += 32) {
        const int x = lo[0] + k / (ny * nz), y = lo[1] + (k / nz) % ny, z = lo[2] + k % nz;
        atomicAdd(t.tcell_count + cell_lin(lay, x, y, z), 1);
    }
}

__global__ void k_tri_fill(Tris t, Grid g)
{
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= t.nt) return;
    if (!tri_range_valid(t, i)) return;
    int lo[3], hi[3];
    const int* lay;
    if (!tri_cell_range(t, g, i, lo, hi, lay)) return;
    const int ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    const int cells = (hi[0] - lo[0] + 1) * ny * nz;
    for (int k = lane; k < cells; k += 32) {
        const int x = lo[0] + k / (ny * nz), y = lo[1] + (k / nz) % ny, z = lo[2] + k % nz;
        const int lin = cell_lin(lay, x, y, z);
        const int pos = t.tcell_start[lin] + atomicAdd(t.tcell_cursor + lin, 1);
        if (pos < t.capacity) { t.ttri_tmp[pos] = i; t.tlin_tmp[pos] = lin; }
        else atomicOr(g.err, kErrTriCapacity);
    }
}

// Triangle-cell entries in ascending triangle order per cell (the order of
// the reference's stable sort of its fill list), placed by rank.
__global__ void k_tri_place(Tris t, Grid g)
{
    const int entries = min(t.tcell_start[*g.total_cells], t.capacity);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < entries; p += gridDim.x * blockDim.x) {
        const int lin = t.tlin_tmp[p];
        const int id = t.ttri_tmp[p];
        const int b = t.tcell_start[lin], e = min(t.tcell_start[lin + 1], t.capacity);
        int rank = 0;
        for (int q = b; q < e; ++q) rank += t.ttri_tmp[q] < id;
        t.ttri[b + rank] = id;
        t.tcell_count[lin] = 0;
        t.tcell_cursor[lin] = 0;
    }
}

// ------------------------------------------------------------ integrator
// quatDerivative / normalizeQuat (src/cuda/cuda_particle_backend.cu:149-183)
__device__ __forceinline__ void quat_derivative(double qw, double qx, double qy, double qz, double wx, double wy,
                                                double wz, double& dw, double& dx, double& dy, double& dz)
{
    dw = 0.5 * fma(-qz, wz, fma(-qy, wy, -qx * wx));
    dx = 0.5 * fma(-qz, wy, fma(qy, wz, qw * wx));
    dy = 0.5 * fma(qz, wx, fma(-qx, wz, qw * wy));
    dz = 0.5 * fma(-qy, wx, fma(qx, wy, qw * wz));
}
// q + quatDerivative(q, w) * h with the derivative's factor 0.5 moved onto
// h: (0.5 s) h and s (0.5 h) are the same product, so the fused result has
// the same bits, without the four multiplications by 0.5.
//
// The quaternion arithmetic here is written with explicit fma: the kernels
// that advance quaternions (a step's finish and advance as two kernels, or
// fused and split around the particle grid) then round alike whatever the
// compiler would contract in each, so a run split into several calls gives
// the bits of one call.
__device__ __forceinline__ void quat_half_step(double& pw, double& px, double& py, double& pz, double wx, double wy,
                                               double wz, double h)
{
    const double qw = pw, qx = px, qy = py, qz = pz, hh = 0.5 * h;
    pw = fma(fma(-qz, wz, fma(-qy, wy, -qx * wx)), hh, pw);
    px = fma(fma(-qz, wy, fma(qy, wz, qw * wx)), hh, px);
    py = fma(fma(qz, wx, fma(-qx, wz, qw * wy)), hh, py);
    pz = fma(fma(-qy, wx, fma(qx, wy, qw * wz)), hh, pz);
}
// 1/sqrt(n2) away from |n2 - 1| < 2^-20, and the reference's degenerate case
// (:170-174); out of line so its FP64 work is issued only by warps that need it.
__device__ __noinline__ double inv_norm_general(double n2) { return n2 <= 1.0e-24 ? 0.0 : rsqrt(n2); }

// A leapfrog quaternion stays within a few ulp of unit length, n2 = 1 + d
// with tiny d, where 1/sqrt(1 + d) = 1 - d/2 + 3d^2/8 - ... : the quadratic
// is exact to below 2^-60 for |d| < 2^-20 (the next term is 5|d|^3/16).  The
// range test reads the exponent of d with integer operations.
__device__ __forceinline__ void normalize_quat(double& qw, double& qx, double& qy, double& qz)
{
    const double n2 = fma(qz, qz, fma(qy, qy, fma(qx, qx, qw * qw)));
    const double d = n2 - 1.0;
    double inv;
    if (((unsigned)__double2hiint(d) & 0x7fffffffu) < 0x3eb00000u) {  // |d| < 2^-20
        inv = fma(d, fma(d, 0.375, -0.5), 1.0);
    } else {
        inv = inv_norm_general(n2);
        if (inv == 0.0) { qw = 1.0; qx = qy = qz = 0.0; return; }
    }
    qw *= inv; qx *= inv; qy *= inv; qz *= inv;
}

// initializeLeapfrogKernel (:185-210)
__global__ void k_leapfrog_init(Owners d, double h)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    d.vhx[i] = d.vx[i] + d.ax[i] * h;
    d.vhy[i] = d.vy[i] + d.ay[i] * h;
    d.vhz[i] = d.vz[i] + d.az[i] * h;
    d.whx[i] = d.wx[i] + d.awx[i] * h;
    d.why[i] = d.wy[i] + d.awy[i] * h;
    d.whz[i] = d.wz[i] + d.awz[i] * h;
    double qw = d.qw[i], qx = d.qx[i], qy = d.qy[i], qz = d.qz[i];
    quat_half_step(qw, qx, qy, qz, d.wx[i], d.wy[i], d.wz[i], h);
    normalize_quat(qw, qx, qy, qz);
    quat_derivative(qw, qx, qy, qz, d.whx[i], d.why[i], d.whz[i], d.hqw[i], d.hqx[i], d.hqy[i], d.hqz[i]);
}

// advancePositionKernel (:212-237)
__global__ void k_advance(Owners d, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n || d.status[i] == -1) return;
    d.px[i] += d.vhx[i] * dt;
    d.py[i] += d.vhy[i] * dt;
    d.pz[i] += d.vhz[i] * dt;
    double qw = fma(d.hqw[i], dt, d.qw[i]), qx = fma(d.hqx[i], dt, d.qx[i]);
    double qy = fma(d.hqy[i], dt, d.qy[i]), qz = fma(d.hqz[i], dt, d.qz[i]);
    normalize_quat(qw, qx, qy, qz);
    d.qw[i] = qw; d.qx[i] = qx; d.qy[i] = qy; d.qz[i] = qz;
    d.vx[i] = d.vhx[i] + d.ax[i] * (0.5 * dt);
    d.vy[i] = d.vhy[i] + d.ay[i] * (0.5 * dt);
    d.vz[i] = d.vhz[i] + d.az[i] * (0.5 * dt);
    d.wx[i] = d.whx[i] + d.awx[i] * (0.5 * dt);
    d.wy[i] = d.why[i] + d.awy[i] * (0.5 * dt);
    d.wz[i] = d.whz[i] + d.awz[i] * (0.5 * dt);
}

// k_advance in two parts, for the first step of a graph-launched run: the
// positions (all the particle grid needs), then the quaternions and the
// full-step velocities beside the grid (grid-stride, two blocks per SM).
__global__ void k_advance_pos(Owners d, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n || d.status[i] == -1) return;
    d.px[i] += d.vhx[i] * dt;
    d.py[i] += d.vhy[i] * dt;
    d.pz[i] += d.vhz[i] * dt;
}
__global__ void __launch_bounds__(256) k_advance_rot(Owners d, double dt)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        if (d.status[i] == -1) continue;
        double qw = fma(d.hqw[i], dt, d.qw[i]), qx = fma(d.hqx[i], dt, d.qx[i]);
        double qy = fma(d.hqy[i], dt, d.qy[i]), qz = fma(d.hqz[i], dt, d.qz[i]);
        normalize_quat(qw, qx, qy, qz);
        d.qw[i] = qw; d.qx[i] = qx; d.qy[i] = qy; d.qz[i] = qz;
        d.vx[i] = d.vhx[i] + d.ax[i] * (0.5 * dt);
        d.vy[i] = d.vhy[i] + d.ay[i] * (0.5 * dt);
        d.vz[i] = d.vhz[i] + d.az[i] * (0.5 * dt);
        d.wx[i] = d.whx[i] + d.awx[i] * (0.5 * dt);
        d.wy[i] = d.why[i] + d.awy[i] * (0.5 * dt);
        d.wz[i] = d.whz[i] + d.awz[i] * (0.5 * dt);
    }
}

// advanceHalfVelocityKernel (:239-265) in its two parts: the half-step
// velocities, then the half-step quaternion rate from the quaternion, the
// full-step spin and the updated half-step spin.
__device__ __forceinline__ void finish_vel_one(Owners d, int i, double dt)
{
    d.vhx[i] += d.ax[i] * dt;
    d.vhy[i] += d.ay[i] * dt;
    d.vhz[i] += d.az[i] * dt;
    d.whx[i] += d.awx[i] * dt;
    d.why[i] += d.awy[i] * dt;
    d.whz[i] += d.awz[i] * dt;
}
__device__ __forceinline__ void finish_rot_one(Owners d, int i, double dt)
{
    const double h = 0.5 * dt;
    double qw = d.qw[i], qx = d.qx[i], qy = d.qy[i], qz = d.qz[i];
    quat_half_step(qw, qx, qy, qz, d.wx[i], d.wy[i], d.wz[i], h);
    normalize_quat(qw, qx, qy, qz);
    quat_derivative(qw, qx, qy, qz, d.whx[i], d.why[i], d.whz[i], d.hqw[i], d.hqx[i], d.hqy[i], d.hqz[i]);
}
__global__ void k_finish(Owners d, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    finish_vel_one(d, i, dt);
    finish_rot_one(d, i, dt);
}
// The parts alone: a run that ends between calls stores the half-step
// velocities and leaves the quaternion rate to the next step's advance
// (k_advance_rest computes it from the same values) or to k_finish_rot,
// whichever comes first.
__global__ void k_finish_vel(Owners d, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.n) finish_vel_one(d, i, dt);
}
__global__ void k_finish_rot(Owners d, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.n) finish_rot_one(d, i, dt);
}

// advanceHalfVelocityKernel of step s followed by advancePositionKernel of
// step s+1, in two parts, so the next step's particle grid (which reads
// positions only) need not wait for the rotational FP64 work.
// Part 1: the half-step velocities of step s and the positions of step s+1.
__global__ void k_finish_advance_pos(Owners d, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const double vhx = d.vhx[i] + d.ax[i] * dt, vhy = d.vhy[i] + d.ay[i] * dt, vhz = d.vhz[i] + d.az[i] * dt;
    d.vhx[i] = vhx; d.vhy[i] = vhy; d.vhz[i] = vhz;
    d.whx[i] += d.awx[i] * dt;
    d.why[i] += d.awy[i] * dt;
    d.whz[i] += d.awz[i] * dt;
    if (d.status[i] == -1) return;
    d.px[i] += vhx * dt;
    d.py[i] += vhy * dt;
    d.pz[i] += vhz * dt;
}

// Part 2 (after part 1): the half-step quaternion rate with the updated
// half-step spin (k_finish's), then the quaternion of step s+1 and its
// full-step velocities (k_advance's), on the values part 1 stored.
__device__ __forceinline__ void advance_rest_one(Owners d, int i, double dt)
{
    const double whx = d.whx[i], why = d.why[i], whz = d.whz[i];
    const double h = 0.5 * dt;
    double qw = d.qw[i], qx = d.qx[i], qy = d.qy[i], qz = d.qz[i];
    double pw = qw, px = qx, py = qy, pz = qz;
    quat_half_step(pw, px, py, pz, d.wx[i], d.wy[i], d.wz[i], h);
    normalize_quat(pw, px, py, pz);
    double hqw, hqx, hqy, hqz;
    quat_derivative(pw, px, py, pz, whx, why, whz, hqw, hqx, hqy, hqz);
    d.hqw[i] = hqw; d.hqx[i] = hqx; d.hqy[i] = hqy; d.hqz[i] = hqz;
    if (d.status[i] == -1) return;
    qw = fma(hqw, dt, qw); qx = fma(hqx, dt, qx); qy = fma(hqy, dt, qy); qz = fma(hqz, dt, qz);
    normalize_quat(qw, qx, qy, qz);
    d.qw[i] = qw; d.qx[i] = qx; d.qy[i] = qy; d.qz[i] = qz;
    d.vx[i] = d.vhx[i] + d.ax[i] * (0.5 * dt);
    d.vy[i] = d.vhy[i] + d.ay[i] * (0.5 * dt);
    d.vz[i] = d.vhz[i] + d.az[i] * (0.5 * dt);
    d.wx[i] = whx + d.awx[i] * (0.5 * dt);
    d.wy[i] = why + d.awy[i] * (0.5 * dt);
    d.wz[i] = whz + d.awz[i] * (0.5 * dt);
}

// One block pair per SM, striding over the owners: the kernel is bound by
// the FP64 pipe, and the particle grid it runs beside takes the other warp
// slots of each SM.
__global__ void __launch_bounds__(256) k_advance_rest(Owners d, double dt)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x)
        advance_rest_one(d, i, dt);
}

// Universal gravitation (src/cuda/cuda_contact_backend.cu:1095-1106): the
// reference adds delta * G m_i m_j / d^3 with delta = p_i - p_j, summed in
// owner order.  Tiled through shared memory, same summation order.
__global__ void k_universal_gravity(Owners o)
{
    __shared__ double sx[256], sy[256], sz[256], sm[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < o.n;
    const double px = act ? o.px[i] : 0.0, py = act ? o.py[i] : 0.0, pz = act ? o.pz[i] : 0.0;
    const double mi = act ? o.mass[i] : 0.0;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int base = 0; base < o.n; base += blockDim.x) {
        const int j = base + threadIdx.x;
        if (j < o.n) { sx[threadIdx.x] = o.px[j]; sy[threadIdx.x] = o.py[j]; sz[threadIdx.x] = o.pz[j]; sm[threadIdx.x] = o.mass[j]; }
        __syncthreads();
        const int lim = min((int)blockDim.x, o.n - base);
        for (int k = 0; k < lim; ++k) {
            if (base + k == i) continue;
            const double dx = px - sx[k], dy = py - sy[k], dz = pz - sz[k];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > 1.0e-28) {
                const double s = kGravityConstant * mi * sm[k] / (d2 * sqrt(d2));
                fx += dx * s; fy += dy * s; fz += dz * s;
            }
        }
        __syncthreads();
    }
    if (act) { o.ugx[i] = fx; o.ugy[i] = fy; o.ugz[i] = fz; }
}

__global__ void k_step_counter(Counters k, int reset)
{
    if (threadIdx.x != 0) return;
    if (reset) {
        *k.pcontacts = 0; *k.phigh = 0; *k.bhigh = 0; *k.ct_total = 0; *k.tgover = 0; *k.wl_total = 0;
        if (k.nl_flag) {
            // an overflowed list is rebuilt by this step's cell sweep
            if (k.nl_flag[1]) k.nl_flag[0] = 1;
            k.nl_flag[1] = 0;
            k.nl_flag[3] = 0;
        }
    } else {
        *k.step += 1;
        if (k.nl_flag) {
            if (k.nl_on && k.nl_flag[0]) k.nl_flag[2] += 1;
            k.nl_flag[0] = 0;
        }
    }
}

inline int blocks(int n, int b) { return (n + b - 1) / b; }

}  // namespace

void launch_update_components(const Comps& c, const Owners& o, cudaStream_t s)
{
    if (c.n > 0) k_update_components<<<blocks(c.n, 256), 256, 0, s>>>(c, o);
}

void launch_scan(const int* in, int* out, const int* n_dev, int* tile_sums, int sm_count, cudaStream_t s)
{
    const int g = sm_count * 2;
    k_scan_reduce<<<g, kScanBlock, 0, s>>>(in, n_dev, tile_sums);
    k_scan_tile_sums<<<1, kScanBlock, 0, s>>>(tile_sums, n_dev);
    k_scan_apply<<<g, kScanBlock, 0, s>>>(in, out, n_dev, tile_sums);
}

__global__ void k_scan_wait_probe(ScanState st, unsigned* err)
{
    // epoch 1: the zero word of tile 0 is never current, so the look-back
    // waits on it until its bound
    (void)scan_lookback(st, 1, 1u, err);
}
void launch_scan_wait_probe(unsigned long long* status, unsigned* err, cudaStream_t s)
{
    ScanState st{status, nullptr, 1};
    k_scan_wait_probe<<<1, 32, 0, s>>>(st, err);
}

void launch_scan1(const int* in, int* out, const int* n_dev, const ScanState& st, unsigned* err, int sm_count,
                  cudaStream_t s)
{
    k_scan1<<<std::max(1, std::min(st.max_tiles, sm_count * 2)), kScan1Block, 0, s>>>(in, out, n_dev, st, err);
}

void launch_grid_layout(const Comps& c, const Owners& o, const Grid& g, cudaStream_t s)
{
    if (c.n <= 0) return;
    k_cell_keys<<<blocks(c.n, 256), 256, 0, s>>>(c, o, g);
    k_layout<<<1, 256, 0, s>>>(g);
}

void launch_grid_sort(const Comps& c, const Owners& o, const Grid& g, int sm_count, cudaStream_t s)
{
    if (c.n <= 0) return;
    k_cell_count<<<blocks(c.n, 256), 256, 0, s>>>(c, o, g);
    launch_scan1(g.cell_count, g.cell_start, g.total_cells, g.scan, g.err, sm_count, s);
    k_scatter<<<blocks(c.n, 256), 256, 0, s>>>(c, g);
    k_place<<<blocks(c.n, 256), 256, 0, s>>>(c, g);
}

void launch_tri_transform(const Tris& t, const Bodies& b, const SceneC* sc, cudaStream_t s)
{
    if (t.nt > 0) k_tri_transform<<<blocks(t.nt, 128), 128, 0, s>>>(t, b, sc);
}

void launch_tri_build(const Tris& t, const Bodies& b, const Grid& g, int* tgover, int sm_count, cudaStream_t s)
{
    if (t.nt <= 0) return;
    k_tri_count<<<blocks(32 * t.nt, 128), 128, 0, s>>>(t, g, tgover);
    launch_scan1(t.tcell_count, t.tcell_start, g.total_cells, t.scan, g.err, sm_count, s);
    k_tri_fill<<<blocks(32 * t.nt, 128), 128, 0, s>>>(t, g);
    k_tri_place<<<sm_count * 8, 256, 0, s>>>(t, g);
}

void launch_universal_gravity(const Owners& o, cudaStream_t s)
{
    if (o.n > 0) k_universal_gravity<<<blocks(o.n, 256), 256, 0, s>>>(o);
}

void launch_leapfrog_init(const Owners& o, double h, cudaStream_t s)
{
    if (o.n > 0) k_leapfrog_init<<<blocks(o.n, 256), 256, 0, s>>>(o, h);
}
void launch_advance(const Owners& o, double dt, cudaStream_t s)
{
    if (o.n > 0) k_advance<<<blocks(o.n, 256), 256, 0, s>>>(o, dt);
}
void launch_advance_pos(const Owners& o, double dt, cudaStream_t s)
{
    if (o.n > 0) k_advance_pos<<<blocks(o.n, 256), 256, 0, s>>>(o, dt);
}
void launch_advance_rot(const Owners& o, double dt, int sm_count, cudaStream_t s)
{
    if (o.n > 0) k_advance_rot<<<std::min(blocks(o.n, 256), 2 * sm_count), 256, 0, s>>>(o, dt);
}
void launch_finish(const Owners& o, double dt, cudaStream_t s)
{
    if (o.n > 0) k_finish<<<blocks(o.n, 256), 256, 0, s>>>(o, dt);
}
void launch_finish_vel(const Owners& o, double dt, cudaStream_t s)
{
    if (o.n > 0) k_finish_vel<<<blocks(o.n, 256), 256, 0, s>>>(o, dt);
}
void launch_finish_rot(const Owners& o, double dt, cudaStream_t s)
{
    if (o.n > 0) k_finish_rot<<<blocks(o.n, 256), 256, 0, s>>>(o, dt);
}
void launch_finish_advance_pos(const Owners& o, double dt, cudaStream_t s)
{
    if (o.n > 0) k_finish_advance_pos<<<blocks(o.n, 256), 256, 0, s>>>(o, dt);
}
void launch_advance_rest(const Owners& o, double dt, int sm_count, cudaStream_t s)
{
    if (o.n > 0) k_advance_rest<<<std::min(blocks(o.n, 256), 2 * sm_count), 256, 0, s>>>(o, dt);
}
void launch_step_counter(const Counters& k, int reset, cudaStream_t s) { k_step_counter<<<1, 32, 0, s>>>(k, reset); }

}  // namespace demgb
