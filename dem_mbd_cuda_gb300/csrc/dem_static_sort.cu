// dem_static_sort.cu -- the cell sort, in a form that allocates nothing.
//
// Some callers cannot call cudaMalloc at the point where they need the
// sorted cell list: code that runs while another component owns all device
// memory through its own pool (a framework's caching allocator, a fixed
// arena sized at start-up), loops with a hard latency budget where a driver
// allocation may stall, and processes with a device-memory quota that is
// already spent.  dem_cell_sort_static gives them the same result as the
// engine's grid build (the reference's sortedCellKey / sortedEntityId):
// packed 63-bit cell keys sorted stably over the input order.  The caller
// passes the device input and output buffers; the working memory comes from
// one file-scope device array (g_sort_scratch) that every GPU which loads
// this library holds until the process exits.
//
// The array's host-side name is only a stand-in for the symbol, not a
// device address: host code looks the address up with cudaGetSymbolAddress
// once per device (with that device current) and passes it to the kernels.
// Every call reuses the same array and leaves its contents behind, so the
// counts are cleared at the start of each call, and calls that overlap on
// the GPU (different streams without ordering, several host threads) race
// on it.
#include "../../include/dem_gb300.h"
#include "dem_kernels.cuh"

#include <climits>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

namespace demgb {
void set_last_error(const std::string& msg);
}

namespace {

using demgb::pack_cell;
using demgb::unpack_cell;

constexpr int kMaxN = DEM_STATIC_SORT_MAX_COMPONENTS;
constexpr int kMaxCells = DEM_STATIC_SORT_MAX_CELLS;
constexpr int kTiles = kMaxCells / 4096 + 64;

// Scratch layout, in ints.
constexpr size_t kOffCount = 0;                                  // kMaxCells + 1
constexpr size_t kOffStart = kOffCount + kMaxCells + 64;         // kMaxCells + 2
constexpr size_t kOffLin = kOffStart + kMaxCells + 64;           // kMaxN
constexpr size_t kOffRank = kOffLin + kMaxN;                     // kMaxN
constexpr size_t kOffTmp = kOffRank + kMaxN;                     // kMaxN
constexpr size_t kOffBox = kOffTmp + kMaxN;                      // 8: box 6, total, err
constexpr size_t kOffTiles = kOffBox + 64;                       // kTiles
constexpr size_t kOffKey = ((kOffTiles + kTiles + 63) / 64) * 64;  // kMaxN uint64 (2 ints each)
constexpr size_t kScratchInts = kOffKey + 2 * (size_t)kMaxN;

static __device__ __align__(256) int g_sort_scratch[kScratchInts];

struct Scratch {
    int *count, *start, *lin, *rank, *tmp, *box, *tiles;
    uint64_t* key;
};

Scratch view(int* base)
{
    Scratch s;
    s.count = base + kOffCount;
    s.start = base + kOffStart;
    s.lin = base + kOffLin;
    s.rank = base + kOffRank;
    s.tmp = base + kOffTmp;
    s.box = base + kOffBox;
    s.tiles = base + kOffTiles;
    s.key = reinterpret_cast<uint64_t*>(base + kOffKey);
    return s;
}

__global__ void k_s_init(Scratch s)
{
    if (threadIdx.x == 0) {
        s.box[0] = s.box[1] = s.box[2] = INT_MAX;
        s.box[3] = s.box[4] = s.box[5] = INT_MIN;
        s.box[6] = 0;  // total cells
        s.box[7] = 0;  // error bits: 1 key range, 2 cell capacity
    }
}

// Cell key per component (computeComponentKeysKernel,
// src/cuda/cuda_grid_backend.cu:51-71) and the cell box.
__global__ void k_s_keys(const double* x, const double* y, const double* z, int n, double inv_mesh, Scratch s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double minCell = -(double)(1 << 20), maxCell = (double)((1 << 20) - 1);
    const double fx = floor(x[i] * inv_mesh), fy = floor(y[i] * inv_mesh), fz = floor(z[i] * inv_mesh);
    if (!isfinite(fx) || !isfinite(fy) || !isfinite(fz) || fx < minCell || fx > maxCell || fy < minCell ||
        fy > maxCell || fz < minCell || fz > maxCell) {
        s.key[i] = 0;
        s.lin[i] = -1;
        atomicOr(s.box + 7, 1);
        return;
    }
    const int cx = (int)fx, cy = (int)fy, cz = (int)fz;
    s.key[i] = pack_cell(cx, cy, cz);
    s.lin[i] = 0;
    atomicMin(s.box + 0, cx); atomicMin(s.box + 1, cy); atomicMin(s.box + 2, cz);
    atomicMax(s.box + 3, cx); atomicMax(s.box + 4, cy); atomicMax(s.box + 5, cz);
}

__global__ void k_s_layout(Scratch s)
{
    if (threadIdx.x != 0) return;
    long long cells = 0;
    if (s.box[0] <= s.box[3]) {
        // each extent is at most 2^21, so the full product can reach 2^63
        // and wrap; it is only formed once the first two extents fit
        const long long nx = (long long)s.box[3] - s.box[0] + 1, ny = (long long)s.box[4] - s.box[1] + 1,
                        nz = (long long)s.box[5] - s.box[2] + 1;
        cells = nx * ny > kMaxCells ? (long long)kMaxCells + 1 : nx * ny * nz;
        if (cells > kMaxCells) {
            s.box[7] |= 2;
            cells = 0;
        }
    }
    s.box[6] = (int)cells;
}

__global__ void k_s_zero(Scratch s)
{
    const int total = s.box[6];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= total; c += gridDim.x * blockDim.x) s.count[c] = 0;
}

__device__ __forceinline__ int s_lin(const int* box, uint64_t key)
{
    int cx, cy, cz;
    unpack_cell(key, cx, cy, cz);
    const int ny = box[4] - box[1] + 1, nz = box[5] - box[2] + 1;
    return ((cx - box[0]) * ny + (cy - box[1])) * nz + (cz - box[2]);
}

__global__ void k_s_count(int n, Scratch s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || s.lin[i] < 0 || s.box[6] == 0) return;
    const int lin = s_lin(s.box, s.key[i]);
    s.lin[i] = lin;
    s.rank[i] = atomicAdd(s.count + lin, 1);
}

__global__ void k_s_scatter(int n, Scratch s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || s.lin[i] < 0 || s.box[6] == 0) return;
    s.tmp[s.start[s.lin[i]] + s.rank[i]] = i;
}

// Rank inside the cell = members with a smaller index: the stable order.
__global__ void k_s_place(int n, Scratch s, uint64_t* sorted_key, int* sorted_id)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || s.lin[i] < 0 || s.box[6] == 0) return;
    const int lin = s.lin[i];
    const int b = s.start[lin], e = s.start[lin + 1];
    int rank = 0;
    for (int p = b; p < e; ++p) rank += s.tmp[p] < i;
    sorted_id[b + rank] = i;
    sorted_key[b + rank] = s.key[i];
}

std::mutex g_setup_mutex;
int* g_device_scratch[64] = {nullptr};

// Once per device, with that device current: the device address of the
// scratch array (the host-side symbol is not a device address).
int* scratch_for_current_device(std::string& err)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return nullptr; }
    if (dev < 0 || dev >= 64) { err = "device ordinal out of range"; return nullptr; }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_device_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess || !p) {
            err = std::string("cudaGetSymbolAddress(g_sort_scratch): ") + cudaGetErrorString(e);
            return nullptr;
        }
        g_device_scratch[dev] = static_cast<int*>(p);
    }
    return g_device_scratch[dev];
}

int fail(int code, const std::string& msg)
{
    demgb::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int dem_cell_sort_static(const double* x, const double* y, const double* z, int n, double mesh_size,
                                    uint64_t* sorted_key, int* sorted_id, void* stream_handle)
{
    if (n < 0) return fail(DEM_ERR_INVALID, "dem_cell_sort_static: negative component count");
    if (n > kMaxN)
        return fail(DEM_ERR_CAPACITY, "dem_cell_sort_static: " + std::to_string(n) +
                                          " components exceed the static scratch limit of " + std::to_string(kMaxN));
    if (!(mesh_size > 0.0)) return fail(DEM_ERR_INVALID, "dem_cell_sort_static: mesh size must be positive");
    if (n == 0) { demgb::set_last_error(""); return DEM_OK; }
    if (!x || !y || !z || !sorted_key || !sorted_id) return fail(DEM_ERR_INVALID, "dem_cell_sort_static: NULL buffer");
    std::string err;
    int* base = scratch_for_current_device(err);
    if (!base) return fail(DEM_ERR_CUDA, err);
    cudaStream_t s = static_cast<cudaStream_t>(stream_handle);
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const Scratch sc = view(base);
    const int blocks = (n + 255) / 256;
    k_s_init<<<1, 32, 0, s>>>(sc);
    k_s_keys<<<blocks, 256, 0, s>>>(x, y, z, n, 1.0 / mesh_size, sc);
    k_s_layout<<<1, 32, 0, s>>>(sc);
    k_s_zero<<<sms * 4, 256, 0, s>>>(sc);
    k_s_count<<<blocks, 256, 0, s>>>(n, sc);
    demgb::launch_scan(sc.count, sc.start, sc.box + 6, sc.tiles, sms, s);
    k_s_scatter<<<blocks, 256, 0, s>>>(n, sc);
    k_s_place<<<blocks, 256, 0, s>>>(n, sc, sorted_key, sorted_id);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DEM_ERR_CUDA, std::string("dem_cell_sort_static launch: ") + cudaGetErrorString(e));
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(DEM_ERR_CUDA, std::string("dem_cell_sort_static: ") + cudaGetErrorString(e));
    int flags = 0;
    e = cudaMemcpy(&flags, base + kOffBox + 7, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(DEM_ERR_CUDA, std::string("dem_cell_sort_static: ") + cudaGetErrorString(e));
    if (flags & 1) return fail(DEM_ERR_CAPACITY, "component grid coordinate exceeds signed 21-bit hash range");
    if (flags & 2)
        return fail(DEM_ERR_CAPACITY, "dem_cell_sort_static: cell box exceeds the static scratch limit of " +
                                          std::to_string(kMaxCells) + " cells");
    demgb::set_last_error("");
    return DEM_OK;
}
