// mavi_noalloc.cu — chunk lists of caller-owned device positions, built
// without allocating device memory (mavi_chunk_lists_noalloc).
//
// Who needs it: a caller that owns every byte of device memory through its
// own pool or budget (a Julia CUDA.jl array pool, a serving process that
// reserved HBM up front) and a caller that must not hit the device-wide
// synchronisation cudaMalloc/cudaFree imply. Such a caller holds positions on
// the device and wants the reference's chunk lists (update_chunks!,
// src/chunks.jl:120-161) without creating a handle, which allocates.
//
// Scratch: one file-scope device array of fixed size (below), located once
// per device with cudaGetSymbolAddress. The array lives in this file's device
// module, which CUDA loads on a device the first time the module is used
// there (lazy loading: the first call of this entry point on that device);
// that load reserves the 4 MiB array and the module's code on the device.
// Later calls allocate nothing. Limits: at most kMaxChunks chunks
// (4 MiB of chunk counters) and a chunk capacity of at most kMaxCap (the
// per-chunk ordering sorts in place). Every call clears the part of the
// scratch it uses on its stream before the first kernel, so nothing has to be
// zero beforehand. All calls on one device share the scratch: calls that
// overlap in time (two host threads, or two streams whose work is in flight
// together) race and produce wrong lists; serialise them per device.
//
// Binning is the same Julia-exact arithmetic the step loop uses, so the lists
// are identical to mavi_get_chunks' for the same positions.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/mavi_cuda.h"
#include "mavi_kernels.cuh"

using namespace mavi;

namespace {

constexpr int64_t kMaxChunks = 1 << 20;                // 1,048,576 chunks
constexpr int64_t kMaxTiles = kMaxChunks / kScanTile;  // 1024 scan tiles
constexpr int32_t kMaxCap = 1024;
constexpr int kMaxDevices = 64;
constexpr int kBlock = 256;

// int32 words: chunk counters | scan-tile totals | error word (DevError)
constexpr int64_t kCountOff = 0;
constexpr int64_t kTileOff = kMaxChunks;
constexpr int64_t kErrOff = kMaxChunks + kMaxTiles;   // 8-byte aligned offset
constexpr int64_t kWords = kErrOff + (int64_t)(sizeof(DevError) / sizeof(int32_t));
static_assert(kErrOff % 2 == 0, "error word must be 8-byte aligned");
static_assert(sizeof(DevError) % sizeof(int32_t) == 0, "error word size");

}  // namespace

static __device__ __align__(256) int32_t g_chunk_scratch[kWords];

// Chunk grid of one replica exactly as mavi_create lays it out (defined in
// mavi_api.cu next to the helpers it uses).
__attribute__((visibility("hidden"))) void replica_chunk_grid(const MaviReplicaParams& p, DevRep& R);

namespace {

std::mutex g_setup_mu;
int32_t* g_scratch_ptr[kMaxDevices] = {};

int say(char* msg, int32_t len, int status, const char* fmt, ...) {
    if (msg && len > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(msg, (size_t)len, fmt, ap);
        va_end(ap);
    }
    return status;
}

// Device address of the scratch array for the current device (set-up on
// first use per device; later calls only read the cached pointer).
int scratch_for_current_device(int32_t** out, char* msg, int32_t len) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return say(msg, len, MAVI_ERR_NO_DEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return say(msg, len, MAVI_ERR_UNSUPPORTED, "device ordinal %d above %d", dev, kMaxDevices - 1);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_chunk_scratch);
        if (e != cudaSuccess || !p)
            return say(msg, len, MAVI_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev,
                       cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<int32_t*>(p);
    }
    *out = g_scratch_ptr[dev];
    return MAVI_OK;
}

__device__ __forceinline__ int64_t cell_of(const DevRep& R, double2 p, DevError* err, int64_t i) {
    int64_t row, col;
    double tx, ty;
    bool finite;
    bin_position(R, p.x, p.y, 0, 0, false, row, col, tx, ty, finite);
    return checked_cell(R, row, col, finite, err, i);   // clamped into the grid; error recorded
}

// Histogram of chunk occupancy plus scan-tile totals (warp-aggregated atomics).
__global__ void k_na_count(const double2* __restrict__ pos, int64_t n, DevRep R, int32_t* __restrict__ count,
                           int32_t* __restrict__ tile_sum, DevError* err) {
    const unsigned full = 0xffffffffu;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = i < n;
    int64_t cell = valid ? cell_of(R, pos[i], err, i) : -1;
    int lane = threadIdx.x & 31;
    unsigned peers = __match_any_sync(full, (int)cell);
    if (valid && lane == __ffs(peers) - 1) {
        int add = __popc(peers);
        int old = atomicAdd(&count[cell], add);
        if (old + add > R.cap) raise_error(err, MAVI_ERR_CHUNK_OVERFLOW, i, cell);
    }
    int tkey = valid ? (int)(cell / kScanTile) : -1;
    unsigned tpeers = __match_any_sync(full, tkey);
    if (valid && lane == __ffs(tpeers) - 1) atomicAdd(&tile_sum[tkey], __popc(tpeers));
}

// Each particle claims a place in its chunk's range; the counters (cleared by
// the scan) serve as cursors. The order inside a chunk is fixed afterwards.
__global__ void k_na_scatter(const double2* __restrict__ pos, int64_t n, DevRep R, int32_t* __restrict__ cursor,
                             const int32_t* __restrict__ start, int32_t* __restrict__ ids, DevError* err) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t cell = cell_of(R, pos[i], err, i);
    int32_t dst = start[cell] + atomicAdd(&cursor[cell], 1);
    if (dst < start[cell + 1]) ids[dst] = (int32_t)i;   // always true: the cursor counts the same particles
}

// Ascending particle id inside each chunk (the order update_chunks! appends
// in, src/chunks.jl:150-161). Chunks above capacity are left unsorted: the
// call reports the overflow.
__global__ void k_na_order(const int32_t* __restrict__ start, int64_t nch, int32_t cap, int32_t* __restrict__ ids) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nch) return;
    int32_t b = start[c], e = start[c + 1];
    if (e - b > cap) return;
    for (int32_t k = b + 1; k < e; k++) {
        int32_t v = ids[k];
        int32_t j = k - 1;
        while (j >= b && ids[j] > v) {
            ids[j + 1] = ids[j];
            j--;
        }
        ids[j + 1] = v;
    }
}

int blocks_for(int64_t n) { return (int)((n + kBlock - 1) / kBlock); }

}  // namespace

extern "C" int mavi_chunk_lists_noalloc(const MaviReplicaParams* params, const double* pos_dev, int64_t n,
                                        int32_t* start_dev, int32_t* ids_dev, void* stream, char* msg,
                                        int32_t msg_len) {
    if (msg && msg_len > 0) msg[0] = '\0';
    if (!params) return say(msg, msg_len, MAVI_ERR_INVALID_ARG, "params is NULL");
    const MaviReplicaParams& p = *params;
    if (p.chunk_rows < 1 || p.chunk_cols < 1)
        return say(msg, msg_len, MAVI_ERR_INVALID_ARG, "chunk_rows and chunk_cols must be >= 1");
    if (p.num_spaces < 1 || p.num_spaces > MAVI_MAX_SPACES)
        return say(msg, msg_len, MAVI_ERR_INVALID_ARG, "num_spaces must be in 1..%d", MAVI_MAX_SPACES);
    if (n < 0 || n > INT32_MAX) return say(msg, msg_len, MAVI_ERR_INVALID_ARG, "n must be in 0..2^31-1");
    const int64_t nch = (int64_t)p.chunk_rows * p.chunk_cols;
    if (nch > kMaxChunks)
        return say(msg, msg_len, MAVI_ERR_INVALID_ARG,
                   "%lld chunks exceed the fixed scratch of mavi_chunk_lists_noalloc (at most %lld chunks)",
                   (long long)nch, (long long)kMaxChunks);
    DevRep R{};
    replica_chunk_grid(p, R);
    if (!(R.chunk_l > 0) || !(R.chunk_h > 0) || !(R.radius > 0))
        return say(msg, msg_len, MAVI_ERR_INVALID_ARG, "degenerate chunk grid or particle radius");
    if (R.cap > kMaxCap || R.cap < 1)
        return say(msg, msg_len, MAVI_ERR_INVALID_ARG,
                   "chunk capacity %d exceeds the limit of mavi_chunk_lists_noalloc (%d)", R.cap, kMaxCap);
    if (!start_dev || (n > 0 && (!pos_dev || !ids_dev)))
        return say(msg, msg_len, MAVI_ERR_INVALID_ARG, "NULL device pointer");
    if ((reinterpret_cast<uintptr_t>(pos_dev) & 15) || (reinterpret_cast<uintptr_t>(start_dev) & 15))
        return say(msg, msg_len, MAVI_ERR_INVALID_ARG, "pos_dev and start_dev must be 16-byte aligned");

    // An error left pending by earlier work of the calling thread is not this
    // call's: report it as such, before anything is launched, instead of
    // attributing it to the launches below (which would also lose it).
    cudaError_t pending = cudaGetLastError();
    if (pending != cudaSuccess)
        return say(msg, msg_len, MAVI_ERR_CUDA,
                   "a CUDA error was pending before this call (not raised by it; now cleared): %s",
                   cudaGetErrorString(pending));
    int32_t* scratch = nullptr;
    int st = scratch_for_current_device(&scratch, msg, msg_len);
    if (st) return st;
    int32_t* count = scratch + kCountOff;
    int32_t* tile_sum = scratch + kTileOff;
    DevError* err = reinterpret_cast<DevError*>(scratch + kErrOff);
    const int64_t ntiles = (nch + kScanTile - 1) / kScanTile;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const double2* pos = reinterpret_cast<const double2*>(pos_dev);

    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int32_t) * nch, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(tile_sum, 0, sizeof(int32_t) * ntiles, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(DevError), s);
    if (e != cudaSuccess) return say(msg, msg_len, MAVI_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    if (n > 0) k_na_count<<<blocks_for(n), kBlock, 0, s>>>(pos, n, R, count, tile_sum, err);
    // k_scan leaves the counters at zero for use as cursors; d_step is unused
    k_scan<<<(unsigned)ntiles, kScanThreads, 0, s>>>(count, nch, tile_sum, start_dev, nullptr, 0);
    if (n > 0) {
        k_na_scatter<<<blocks_for(n), kBlock, 0, s>>>(pos, n, R, count, start_dev, ids_dev, err);
        k_na_order<<<blocks_for(nch), kBlock, 0, s>>>(start_dev, nch, R.cap, ids_dev);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return say(msg, msg_len, MAVI_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
    DevError h{};
    e = cudaMemcpyAsync(&h, err, sizeof(DevError), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return say(msg, msg_len, MAVI_ERR_CUDA, "%s", cudaGetErrorString(e));
    switch (h.code) {
    case 0: return MAVI_OK;
    case MAVI_ERR_OUT_OF_GRID:
        return say(msg, msg_len, h.code, "particle %d is outside the chunk grid (row*1000003+col = %lld)", h.slot,
                   (long long)h.aux);
    case MAVI_ERR_CHUNK_OVERFLOW:
        return say(msg, msg_len, h.code, "chunk %lld holds more particles than its capacity %d", (long long)h.aux,
                   R.cap);
    case MAVI_ERR_NONFINITE:
        return say(msg, msg_len, h.code, "particle %d has a non-finite position", h.slot);
    }
    return say(msg, msg_len, h.code, "device error %d", h.code);
}
