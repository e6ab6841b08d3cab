// hgpu_noalloc.cu -- self-annihilation of a spawned list without any device
// allocation by the library.
//
// Who needs this: a host program that owns every byte of device memory through
// its own pool allocator (and so can hand the library its input and output
// buffers, but cannot let the library call cudaMalloc behind its back), and a
// caller on a latency-critical path that must not allocate at all, because
// cudaMalloc and cudaFree can synchronise the whole device.  The entry point
// works only inside buffers the caller passes plus a fixed scratch area that
// is part of the library image itself.
//
// The scratch area is the file-scope device array g_noalloc_scratch below.  Its
// size is fixed at kNoallocBytes (about 5 MB): every GPU that loads the library
// holds it until the process exits, whether or not this entry point is called.
// Host code must not use the array's name as an address (on the host it names
// a host-side placeholder); the device address is obtained once per device with
// cudaGetSymbolAddress, on the first call made with that device current, and
// kept for the life of the process: after a cudaDeviceReset (which destroys the
// primary context and with it the module's memory) the kept address is stale,
// so a reset between calls is not supported.  All calls share the one array:
// two calls whose work overlaps on the GPU (for example on two streams) race
// and corrupt each other's results, so callers must order them.
//
// The operation is HANDE's annihilate_spawn_t (src/spawn_data.F90:859-935)
// after the qsort of annihilate_wrapper_spawn_t_single (:406): sort the entries
// by determinant (unsigned, last word most significant), add the populations
// of equal determinants, drop the determinants whose populations all cancel.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/hande_gpu.h"
#include "hgpu_device.cuh"

namespace {

using namespace hgpu;

constexpr int64_t kNoallocMaxEntries = HGPU_NOALLOC_MAX_ENTRIES;
constexpr int kNaBlock = 256;
constexpr int kNaGrid = 64;  // blocks of the radix and reduction kernels
constexpr int kNaRadix = 256;

// Byte layout of the scratch area (offsets are multiples of 256).
constexpr size_t kKeyBytes = (size_t)kNoallocMaxEntries * 8 * HGPU_MAX_WORDS;  // one key buffer
constexpr size_t kIdxBytes = (size_t)kNoallocMaxEntries * 4;
constexpr size_t kOffKeys0 = 0;
constexpr size_t kOffKeys1 = kOffKeys0 + kKeyBytes;
constexpr size_t kOffIdx0 = kOffKeys1 + kKeyBytes;
constexpr size_t kOffIdx1 = kOffIdx0 + kIdxBytes;
constexpr size_t kOffHist = kOffIdx1 + kIdxBytes;                       // kNaRadix * kNaGrid u32
constexpr size_t kOffKeep = kOffHist + (size_t)kNaRadix * kNaGrid * 4;  // u32 per entry
constexpr size_t kOffPos = kOffKeep + kIdxBytes;                        // u32 exclusive scan
constexpr size_t kOffCount = kOffPos + kIdxBytes;                       // int64 result count
constexpr size_t kNoallocBytes = kOffCount + 256;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

struct Scratch {
    uint64_t *keys[2];
    uint32_t *idx[2];
    uint32_t *hist;
    uint32_t *keep;
    uint32_t *pos;
    int64_t *count;
};

Scratch carve(unsigned char *base) {
    Scratch s;
    s.keys[0] = reinterpret_cast<uint64_t *>(base + kOffKeys0);
    s.keys[1] = reinterpret_cast<uint64_t *>(base + kOffKeys1);
    s.idx[0] = reinterpret_cast<uint32_t *>(base + kOffIdx0);
    s.idx[1] = reinterpret_cast<uint32_t *>(base + kOffIdx1);
    s.hist = reinterpret_cast<uint32_t *>(base + kOffHist);
    s.keep = reinterpret_cast<uint32_t *>(base + kOffKeep);
    s.pos = reinterpret_cast<uint32_t *>(base + kOffPos);
    s.count = reinterpret_cast<int64_t *>(base + kOffCount);
    return s;
}

__device__ __forceinline__ void na_range(int64_t n, int64_t &b, int64_t &e) {
    int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    b = (int64_t)blockIdx.x * chunk;
    e = b + chunk < n ? b + chunk : n;
    if (b > n) b = n;
}

// Keys of the entries: the determinant words of sdata(nw+R+1, n).
__global__ void k_na_keys(const int64_t *sdata, int64_t n, int nw, int el, uint64_t *keys) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int k = 0; k < nw; k++) keys[i * nw + k] = (uint64_t)sdata[i * el + k];
}

__global__ void k_na_hist(const uint64_t *keys, int64_t n, int nw, int shift, uint32_t *hist) {
    __shared__ uint32_t h[kNaRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t b, e;
    na_range(n, b, e);
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x)
        atomicAdd(&h[(keys[i * nw + (shift >> 6)] >> (shift & 63)) & (kNaRadix - 1)], 1u);
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan, in place, of a short array (one block).
__global__ void k_na_scan(uint32_t *a, int64_t len, int64_t *total) {
    __shared__ uint32_t carry, wsum[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t base = 0; base < len; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        uint32_t v = i < len ? a[i] : 0u;
        uint32_t x = v;
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < nw ? wsum[lane] : 0u;
            for (int d = 1; d < 32; d <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d) w += y;
            }
            if (lane < nw) wsum[lane] = w;
        }
        __syncthreads();
        uint32_t before = (warp > 0 ? wsum[warp - 1] : 0u) + carry;
        if (i < len) a[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

// Stable scatter of one radix pass: each block walks its chunk in order, one
// warp at a time, so equal digits keep their input order.
__global__ void k_na_scatter(const uint64_t *kin, const uint32_t *iin, uint64_t *kout, uint32_t *iout, int64_t n,
                             int nw, int shift, const uint32_t *hist) {
    __shared__ uint32_t off[kNaRadix];
    off[threadIdx.x] = hist[threadIdx.x * gridDim.x + blockIdx.x];
    __syncthreads();
    int64_t b, e;
    na_range(n, b, e);
    if (threadIdx.x >= 32) return;  // one warp keeps the order
    int lane = threadIdx.x;
    for (int64_t base = b; base < e; base += 32) {
        int64_t i = base + lane;
        bool valid = i < e;
        uint32_t mask = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            uint32_t d = (uint32_t)((kin[i * nw + (shift >> 6)] >> (shift & 63)) & (kNaRadix - 1));
            uint32_t peers = __match_any_sync(mask, d);
            int leader = __ffs(peers) - 1;
            uint32_t lt = (1u << lane) - 1u;
            uint32_t rank = __popc(peers & lt);
            uint32_t basepos = 0;
            if (lane == leader) {
                basepos = off[d];
                off[d] = basepos + __popc(peers);
            }
            basepos = __shfl_sync(mask, basepos, leader);
            uint32_t p = basepos + rank;
            for (int k = 0; k < nw; k++) kout[(int64_t)p * nw + k] = kin[i * nw + k];
            iout[p] = iin ? iin[i] : (uint32_t)i;
        }
        __syncwarp();
    }
}

// Heads of equal-determinant runs sum their run; keep[] marks non-zero sums.
__global__ void k_na_reduce(const uint64_t *keys, const uint32_t *idx, const int64_t *sdata, int64_t n, int nw,
                            int R, int el, uint32_t *keep) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        bool head = true;
        if (i > 0) {
            head = false;
            for (int k = 0; k < nw; k++) head = head || keys[i * nw + k] != keys[(i - 1) * nw + k];
        }
        if (!head) {
            keep[i] = 0;
            continue;
        }
        bool nz = false;
        for (int q = 0; q < R; q++) {
            int64_t s = 0;
            for (int64_t j = i; j < n; j++) {
                bool same = true;
                for (int k = 0; k < nw; k++) same = same && keys[j * nw + k] == keys[i * nw + k];
                if (!same) break;
                s += sdata[(int64_t)idx[j] * el + nw + q];
            }
            nz = nz || s != 0;
        }
        keep[i] = nz ? 1u : 0u;
    }
}

// Write the surviving determinants and their summed populations: out(nw+R, m).
__global__ void k_na_write(const uint64_t *keys, const uint32_t *idx, const int64_t *sdata, const uint32_t *keep,
                           const uint32_t *pos, int64_t n, int nw, int R, int el, int64_t *out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        int64_t o = (int64_t)pos[i] * (nw + R);
        for (int k = 0; k < nw; k++) out[o + k] = (int64_t)keys[i * nw + k];
        for (int q = 0; q < R; q++) {
            int64_t s = 0;
            for (int64_t j = i; j < n; j++) {
                bool same = true;
                for (int k = 0; k < nw; k++) same = same && keys[j * nw + k] == keys[i * nw + k];
                if (!same) break;
                s += sdata[(int64_t)idx[j] * el + nw + q];
            }
            out[o + nw + q] = s;
        }
    }
}

std::mutex g_setup_lock;
unsigned char *g_scratch_dev[64];  // device address of the scratch area, per device ordinal

}  // namespace

extern "C" int32_t hgpu_self_annihilate_noalloc(const int64_t *d_sdata, int64_t n, int32_t nwords, int32_t nspaces,
                                                int64_t *d_out, int64_t *n_out, void *stream) {
    if (!n_out || nwords < 1 || nwords > HGPU_MAX_WORDS || nspaces < 1 || nspaces > HGPU_MAX_SPACES || n < 0 ||
        (n > 0 && (!d_sdata || !d_out)))
        return HGPU_ERR_INVALID;
    if (n > kNoallocMaxEntries) {
        // too large for the fixed scratch area: say so through the count
        *n_out = -kNoallocMaxEntries;
        return HGPU_ERR_INVALID;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return HGPU_ERR_NO_DEVICE;
    }
    unsigned char *base;
    {
        // first call on this device: look up the device address of the scratch
        // array, with this device current
        std::lock_guard<std::mutex> lk(g_setup_lock);
        if (!g_scratch_dev[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return HGPU_ERR_CUDA;
            }
            g_scratch_dev[dev] = static_cast<unsigned char *>(p);
        }
        base = g_scratch_dev[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch s = carve(base);
    int W = nwords, R = nspaces, el = W + R + 1;
    // the result count starts at zero for an empty list
    if (cudaMemsetAsync(s.count, 0, sizeof(int64_t), st) != cudaSuccess) goto cuda_fail;
    if (n > 0) {
        k_na_keys<<<kNaGrid, kNaBlock, 0, st>>>(d_sdata, n, W, el, s.keys[0]);
        const uint32_t *iin = nullptr;
        int cur = 0;
        int passes = 64 * W / 8;
        for (int p = 0; p < passes; p++) {
            int shift = 8 * p;
            k_na_hist<<<kNaGrid, kNaRadix, 0, st>>>(s.keys[cur], n, W, shift, s.hist);
            k_na_scan<<<1, 1024, 0, st>>>(s.hist, (int64_t)kNaRadix * kNaGrid, nullptr);
            k_na_scatter<<<kNaGrid, kNaRadix, 0, st>>>(s.keys[cur], iin, s.keys[1 - cur], s.idx[1 - cur], n, W, shift,
                                                       s.hist);
            iin = s.idx[1 - cur];
            cur = 1 - cur;
        }
        k_na_reduce<<<kNaGrid, kNaBlock, 0, st>>>(s.keys[cur], s.idx[cur], d_sdata, n, W, R, el, s.keep);
        // positions: exclusive scan of keep (copied, then scanned in place)
        if (cudaMemcpyAsync(s.pos, s.keep, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            goto cuda_fail;
        k_na_scan<<<1, 1024, 0, st>>>(s.pos, n, s.count);
        k_na_write<<<kNaGrid, kNaBlock, 0, st>>>(s.keys[cur], s.idx[cur], d_sdata, s.keep, s.pos, n, W, R, el, d_out);
    }
    if (cudaMemcpyAsync(n_out, s.count, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess) goto cuda_fail;
    if (cudaStreamSynchronize(st) != cudaSuccess) goto cuda_fail;
    return HGPU_OK;
cuda_fail:
    cudaGetLastError();
    return HGPU_ERR_CUDA;
}
